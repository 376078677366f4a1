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
