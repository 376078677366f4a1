"""Batched waves and the render server: a job's image is the same alone and in
the mix (bit for bit), admission respects the memory budget, and camera
overrides render like a scene created with that camera."""
import numpy as np
import pytest

import gr
from gr import scenes as sc

pytestmark = pytest.mark.gpu


def _small_jobs():
    jobs = []
    d = sc.cornell_box(48, 40)
    jobs.append((d, dict(spp=6, max_depth=8, seed=1)))
    g = sc.glossy_scene(64, 48, level=3, glass_level=2)
    jobs.append((g, dict(spp=4, max_depth=12, seed=2, rr_depth=3)))
    j3, _ = sc.batch_job(5, min_tris=2000, max_tris=30000)
    j3.camera = dict(j3.camera, width=40, height=40)
    jobs.append((j3, dict(spp=5, max_depth=8, seed=3)))
    return jobs


def _alone(ctx, desc, o):
    s = gr.Scene(ctx, desc)
    s.render(o["spp"], o.get("max_depth", 8), o.get("seed", 0), o.get("rr_depth", 3), o.get("flags", 0),
             want_image=False)
    return s


def test_batch_equals_alone(ctx):
    jobs = _small_jobs()
    alone = [_alone(ctx, d, o).accumulation() for d, o in jobs]
    scenes = [gr.Scene(ctx, d) for d, _ in jobs]
    # a small wave forces jobs to share and split waves
    st = gr.render_batch(ctx, scenes, [o for _, o in jobs], wave_paths=3000)
    assert st.waves > 1 and st.device_errors == 0
    for s, (sa, ca) in zip(scenes, alone):
        sb, cb = s.accumulation()
        np.testing.assert_array_equal(cb, ca)
        np.testing.assert_array_equal(sb, sa)


def test_batch_rejects_duplicate_scene(ctx):
    d = sc.cornell_box(16, 16)
    s = gr.Scene(ctx, d)
    with pytest.raises(gr.GrError):
        gr.render_batch(ctx, [s, s], [dict(spp=1), dict(spp=1)])


def test_server_results_equal_alone(ctx):
    jobs = _small_jobs()
    srv = gr.Server(ctx, wave_paths=5000)
    scenes = [gr.Scene(ctx, d) for d, _ in jobs]
    tickets = []
    for rep in range(2):  # every scene twice: repeated scene ids share the resident BVH
        for s, (d, o) in zip(scenes, jobs):
            tickets.append((srv.submit(s, o["spp"], o.get("max_depth", 8), o.get("seed", 0), o.get("rr_depth", 3)),
                            d, o))
    for t, d, o in tickets:
        done, img, js = srv.wait(t, timeout=60.0, image_shape=(d.camera["height"], d.camera["width"]))
        assert done and js.status == 0
        ref, _ = _alone(ctx, d, o).render(0, want_image=True)
        np.testing.assert_array_equal(img, ref)
        assert js.submit_s <= js.admit_s <= js.done_s
    st = srv.stats()
    assert st.completed == len(tickets) and st.waves >= 1
    srv.close()


def test_server_budget_admission(ctx):
    d = sc.cornell_box(64, 64)
    s = gr.Scene(ctx, d)
    budget_probe = gr.Server(ctx, wave_paths=64 * 64 * 4)
    base = budget_probe.stats().bytes_in_use
    budget_probe.close()
    scene_bytes = gr._declare(gr._SERVER_SIGS).gr_scene_device_bytes(s.h)
    per_job = 64 * 64 * 28
    # room for the scene and one job at a time
    srv = gr.Server(ctx, budget_bytes=base + scene_bytes + per_job + 16, wave_paths=64 * 64 * 4)
    ts = [srv.submit(s, 4, 8, seed=k) for k in range(4)]
    res = [srv.wait(t, timeout=60.0, image_shape=(64, 64)) for t in ts]
    assert all(r[0] for r in res)
    st = srv.stats()
    assert st.peak_bytes <= base + scene_bytes + per_job + 16
    # one at a time: each job is admitted after the previous finished
    for a, b in zip(res, res[1:]):
        assert b[2].admit_s >= a[2].done_s - 1e-3
    for k, r in enumerate(res):
        ref, _ = _alone(ctx, d, dict(spp=4, max_depth=8, seed=k)).render(0)
        np.testing.assert_array_equal(r[1], ref)
    srv.close()


def test_server_camera_override(ctx):
    d = sc.cornell_box(32, 32)
    s = gr.Scene(ctx, d)
    cam2 = dict(d.camera, width=24, height=20, fov=50.0)
    srv = gr.Server(ctx)
    t = srv.submit(s, 4, 6, seed=9, camera=cam2)
    done, img, _ = srv.wait(t, timeout=60.0, image_shape=(20, 24))
    srv.close()
    d2 = sc.cornell_box(32, 32)
    d2.camera = cam2
    ref, _ = _alone(ctx, d2, dict(spp=4, max_depth=6, seed=9)).render(0)
    np.testing.assert_array_equal(img, ref)


def test_server_poll_reports_like_wait(ctx):
    """gr_server_poll: not done while the job runs (or done at once), then done
    with the same image a plain render gives; a finished ticket is reported once."""
    import time
    d, o = _small_jobs()[0]
    srv = gr.Server(ctx, wave_paths=5000)
    s = gr.Scene(ctx, d)
    t = srv.submit(s, o["spp"], o.get("max_depth", 8), o.get("seed", 0), o.get("rr_depth", 3))
    shape = (d.camera["height"], d.camera["width"])
    deadline = time.time() + 60.0
    while True:
        done, img, js = srv.poll(t, image_shape=shape)
        if done or time.time() > deadline:
            break
        time.sleep(0.001)
    assert done and js.status == 0
    ref, _ = _alone(ctx, d, o).render(0, want_image=True)
    np.testing.assert_array_equal(img, ref)
    with pytest.raises(gr.GrError):
        srv.poll(t)
    srv.close()


def test_server_wave_failure_fails_jobs_and_returns(ctx):
    """Host-side fault injection (nothing faults on the GPU): a wave that
    reports a failed launch ends every job in flight with GR_ERR_CUDA; waiting
    on them returns at once, later jobs render normally, and destroying the
    server returns with jobs still queued."""
    d, o = _small_jobs()[0]
    s = gr.Scene(ctx, d)
    shape = (d.camera["height"], d.camera["width"])
    srv = gr.Server(ctx, wave_paths=5000)
    srv.fail_waves(1)
    t_bad = srv.submit(s, o["spp"], 8, seed=1)
    with pytest.raises(gr.GrError) as e:
        srv.wait(t_bad, timeout=-1.0)  # a wait with no timeout must come back
    assert e.value.status == gr.GR_ERR_CUDA
    t_ok = srv.submit(s, o["spp"], 8, seed=1)
    done, img, js = srv.wait(t_ok, timeout=60.0, image_shape=shape)
    assert done and js.status == 0
    ref, _ = _alone(ctx, d, dict(spp=o["spp"], max_depth=8, seed=1)).render(0)
    np.testing.assert_array_equal(img, ref)
    # every wave fails from here on: queued jobs fail too, and destroy returns
    srv.fail_waves(1 << 30)
    ts = [srv.submit(s, 4, 8, seed=k) for k in range(3)]
    for t in ts:
        with pytest.raises(gr.GrError):
            srv.wait(t, timeout=-1.0)
    srv.submit(s, 4, 8, seed=7)
    srv.close()


def test_server_admits_a_job_mid_flight_and_shares_waves(ctx):
    """Continuous batching: job B, submitted while job A is on the GPU, is
    admitted before A finishes and runs in waves A also runs in; both images
    equal the same jobs rendered alone."""
    import time
    da = sc.cornell_box(160, 120)
    db = sc.cornell_box(48, 40, seed_salt=3)
    sa, sb = gr.Scene(ctx, da), gr.Scene(ctx, db)
    # a wave holds two of A's samples (A needs 256 waves) and room for all of B's
    srv = gr.Server(ctx, wave_paths=160 * 120 * 2 + 48 * 40 * 8)
    ta = srv.submit(sa, 512, 8, seed=4)
    deadline = time.time() + 30.0
    while srv.stats().waves < 4 and time.time() < deadline:  # A is running
        time.sleep(0.0005)
    tb = srv.submit(sb, 8, 8, seed=5)
    done_b, img_b, jb = srv.wait(tb, timeout=60.0, image_shape=(40, 48))
    done_a, img_a, ja = srv.wait(ta, timeout=120.0, image_shape=(120, 160))
    assert done_a and done_b and ja.status == 0 and jb.status == 0
    assert jb.admit_s < ja.done_s
    assert ja.first_wave < jb.first_wave <= jb.last_wave <= ja.last_wave  # B ran inside A's run of waves
    assert jb.waves >= 1 and ja.waves >= 2
    np.testing.assert_array_equal(img_a, _alone(ctx, da, dict(spp=512, max_depth=8, seed=4)).render(0)[0])
    np.testing.assert_array_equal(img_b, _alone(ctx, db, dict(spp=8, max_depth=8, seed=5)).render(0)[0])
    srv.close()


def test_server_shortest_first_lets_small_jobs_pass(ctx):
    """GR_SERVER_SHORTEST_FIRST: small jobs submitted after a large one finish
    before it. First come first served (or shortest first with an age cap every
    job has already passed) keeps the large job ahead: the wave is full of its
    samples until it is done."""
    big = sc.cornell_box(160, 120)
    small = sc.cornell_box(32, 32, seed_salt=1)
    sbig, ssmall = gr.Scene(ctx, big), gr.Scene(ctx, small)
    for policy, age_cap, small_first in ((gr.SERVER_SHORTEST_FIRST, 0.0, True), (gr.SERVER_FIFO, 0.0, False),
                                         (gr.SERVER_SHORTEST_FIRST, 1e-9, False)):
        srv = gr.Server(ctx, wave_paths=160 * 120 * 2, policy=policy, age_cap_s=age_cap)
        tb = srv.submit(sbig, 256, 8, seed=1)
        ts = [srv.submit(ssmall, 4, 8, seed=10 + k) for k in range(4)]
        rs = [srv.wait(t, timeout=60.0, image_shape=(32, 32)) for t in ts]
        rb = srv.wait(tb, timeout=120.0, image_shape=(120, 160))
        last_small = max(r[2].done_s for r in rs)
        if small_first:
            assert last_small < rb[2].done_s
        else:
            assert min(r[2].done_s for r in rs) >= rb[2].done_s - 1e-3
        for k, r in enumerate(rs):  # the order does not change any image
            np.testing.assert_array_equal(r[1], _alone(ctx, small, dict(spp=4, max_depth=8, seed=10 + k)).render(0)[0])
        srv.close()


def test_server_load_shedding_refuses_what_it_cannot_start(ctx):
    """max_wait_s: once the server has measured its throughput, a job whose
    queued work ahead would take longer than the limit is refused with
    GR_ERR_BUSY (counted in stats.rejected); accepted jobs complete."""
    d = sc.cornell_box(128, 128)
    s = gr.Scene(ctx, d)
    srv = gr.Server(ctx, wave_paths=128 * 128 * 4, max_wait_s=0.05)
    t0 = srv.submit(s, 16, 8, seed=0)
    assert srv.wait(t0, timeout=60.0)[0]  # throughput now measured
    accepted, refused = [], 0
    for k in range(400):  # far more work than 50 ms of rendering
        try:
            accepted.append(srv.submit(s, 64, 8, seed=k + 1))
        except gr.GrError as e:
            assert e.status == gr.GR_ERR_BUSY
            refused += 1
    assert refused > 0 and srv.stats().rejected == refused
    for t in accepted:
        assert srv.wait(t, timeout=120.0)[0]
    srv.close()
