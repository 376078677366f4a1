"""Timed workloads for the render configurations (used by bench.py).

config 1: plain render of the procedural Cornell box, 256x256, 16 spp, depth 8.
config 3: plain render of the glossy scene, 1024x768, 64 spp, depth 16, RR after 3.
config 4: 64 seeded jobs (10k-2M triangles, 128^2..1024^2, 4/16/64 spp, depth 8)
          rendered one gr_render call after another, then all in gr_render_batch.
config 5: Poisson arrivals of config-4-distributed requests served by gr_server
          (continuous batching, HBM budget, resident BVHs per scene id), with
          p50/p99 latency, against the same stream served one job at a time.
"""
import threading
import time

import numpy as np

import gr
from gr import scenes as sc


def _timed_render(scene, spp, depth, rr=3, flags=0, reps=3):
    scene.render(spp, depth, 1, rr, flags, want_image=False)
    best = None
    st = None
    for _ in range(reps):
        scene.reset()
        t = time.perf_counter()
        _, st = scene.render(spp, depth, 1, rr, flags, want_image=False)
        dt = time.perf_counter() - t
        best = dt if best is None else min(best, dt)
    return best, st


def _names():
    return {v: k for k, v in gr.LAYOUT_NAMES.items()}


def tuning_args(tune, wave=0):
    """(layout, block, short_stack, wave_paths) from an autotuner result."""
    return (_names()[tune["layout"]], tune["block"], tune["short_stack"], wave)


def plain_render(ctx, desc, spp, depth, rr=3, autotune=True, tuning=None):
    """One scene rendered by gr_render; with autotune the scene's traversal
    configuration and wave size come from gr_scene_autotune (1-spp probes),
    else from `tuning` = (layout, block, short_stack, wave_paths) if given."""
    s = gr.Scene(ctx, desc)
    if tuning is not None:
        s.set_tuning(*tuning)
    if autotune:
        s.autotune(spp=1, max_depth=depth, rr_depth=rr)
    dt, st = _timed_render(s, spp, depth, rr)
    npix = desc.camera["width"] * desc.camera["height"]
    out = {"ms": dt * 1e3, "samples_per_s": npix * spp / dt, "mrays_s": (st.closest_rays + st.shadow_rays) / dt / 1e6,
           "triangles": desc.num_triangles, "waves": st.waves, "tuning": s.tuning()[0], "wave_paths": s.tuning()[1]}
    s.close()
    return out


def config4(ctx, n_jobs=64, autotune=True):
    """Returns renders/s of the 64-job stream rendered the reference's way (one
    frame per sample per scene), as one multi-sample gr_render per scene, and
    as one gr_render_batch: once with the default traversal configuration
    (binary nodes, 128-thread blocks, 12-entry shared stack, 4 Mi-path waves)
    and once with the configuration and wave size gr_scene_autotune picks on
    the job with the most samples. Images are identical in all modes and
    configurations, so RMSE is equal by construction."""
    jobs = [sc.batch_job(i) for i in range(n_jobs)]
    scenes = [gr.Scene(ctx, d) for d, _ in jobs]
    opts = [dict(spp=spp, max_depth=8, seed=i) for i, (_, spp) in enumerate(jobs)]
    samples = sum(d.camera["width"] * d.camera["height"] * spp for d, spp in jobs)
    out = {"jobs": n_jobs, "triangles": sum(d.num_triangles for d, _ in jobs), "samples": samples}
    modes = [("default", (gr.LAYOUT_BVH2, 128, 12, 0))]
    if autotune:
        big = max(range(n_jobs), key=lambda i: jobs[i][0].camera["width"] * jobs[i][0].camera["height"] * jobs[i][1])
        t0 = time.perf_counter()
        tune, wave = scenes[big].autotune(spp=1, max_depth=8)
        out["autotune"] = {"probe_job": big, "tuning": tune, "wave_paths": wave,
                           "seconds": time.perf_counter() - t0}
        modes.append(("autotuned", tuning_args(tune, wave)))
    for name, (layout, block, sstack, wave) in modes:
        for s in scenes:
            s.set_tuning(layout, block, sstack, wave)
        # warm-up: one small render per scene (captures graphs, touches memory)
        for s in scenes:
            s.render(1, 8, 0, want_image=False)
            s.reset()
        gr.render_batch(ctx, scenes, [dict(spp=1, max_depth=8)] * len(scenes), wave_paths=wave)
        for s in scenes:
            s.reset()
        t = time.perf_counter()
        rays = 0
        for s, o in zip(scenes, opts):
            _, st = s.render(o["spp"], 8, o["seed"], want_image=False)
            rays += st.closest_rays + st.shadow_rays
        t_seq = time.perf_counter() - t
        # the reference's schedule: one frame (1 spp) per render() call, launched
        # kernel by kernel and waited for (PathTracer::render(num), pathtracer.cu:152-170)
        for s in scenes:
            s.reset()
        t = time.perf_counter()
        for s, o in zip(scenes, opts):
            for _ in range(o["spp"]):
                s.render(1, 8, o["seed"], flags=gr.RENDER_NO_GRAPH, want_image=False)
        t_frames = time.perf_counter() - t
        for s in scenes:
            s.reset()
        t = time.perf_counter()
        st = gr.render_batch(ctx, scenes, opts, wave_paths=wave)
        t_batch = time.perf_counter() - t
        out[name] = {"tuning": scenes[0].tuning()[0], "wave_paths": wave or (1 << 22),
                     "per_frame_renders_s": n_jobs / t_frames, "sequential_renders_s": n_jobs / t_seq,
                     "batched_renders_s": n_jobs / t_batch, "speedup_vs_per_frame": t_frames / t_batch,
                     "speedup_vs_sequential": t_seq / t_batch, "per_frame_s": t_frames, "sequential_s": t_seq,
                     "batched_s": t_batch, "batched_mrays_s": (st.closest_rays + st.shadow_rays) / t_batch / 1e6,
                     "sequential_mrays_s": rays / t_seq / 1e6, "batched_waves": st.waves}
    for s in scenes:
        s.close()
    return out


def _serve(ctx, scenes, requests, budget, max_active, rate, tuning, policy=gr.SERVER_FIFO, age_cap_s=0.0,
           max_wait_s=0.0):
    """Submits `requests` (scene index, camera, spp, seed) at Poisson times of
    `rate` per second; returns latency and throughput figures. With
    max_wait_s > 0 the server refuses requests it cannot start in time
    (GR_ERR_BUSY); those count as rejected and have no latency."""
    layout, block, sstack, wave = tuning
    srv = gr.Server(ctx, budget_bytes=budget, wave_paths=wave, max_active=max_active, layout=layout, block=block,
                    short_stack=sstack, policy=policy, age_cap_s=age_cap_s, max_wait_s=max_wait_s)
    r = np.random.default_rng(12345)
    gaps = r.exponential(1.0 / rate, size=len(requests))
    tickets = []
    rejected = 0
    t0 = time.perf_counter()
    t_next = t0
    for (si, cam, spp, seed), gap in zip(requests, gaps):
        t_next += gap
        delay = t_next - time.perf_counter()
        if delay > 0:
            time.sleep(delay)
        try:
            tickets.append(srv.submit(scenes[si], spp, 8, seed, camera=cam))
        except gr.GrError as e:
            if e.status != gr.GR_ERR_BUSY:
                raise
            rejected += 1
    offered_s = time.perf_counter() - t0
    lat, done_s, sub_s = [], [], []
    samples = 0
    for t in tickets:
        ok, _, js = srv.wait(t, timeout=900.0)
        if ok:
            lat.append(js.done_s - js.submit_s)
            done_s.append(js.done_s)
            sub_s.append(js.submit_s)
            samples += js.samples
    st = srv.stats()
    srv.close()
    span = max(done_s) - min(sub_s) if done_s else float("nan")
    lat = np.asarray(lat) if lat else np.asarray([float("nan")])
    return {"rate": rate, "requests": len(requests), "completed": len(done_s), "rejected": rejected,
            "offered_s": offered_s, "p50_ms": float(np.percentile(lat, 50) * 1e3),
            "p99_ms": float(np.percentile(lat, 99) * 1e3), "max_ms": float(np.max(lat) * 1e3),
            "renders_s": len(done_s) / span, "msamples_s": samples / span / 1e6, "waves": int(st.waves),
            "peak_bytes": int(st.peak_bytes)}


def config5_sweep(ctx, rates=(10, 20, 50, 100, 200, 500), window_s=20.0, fifo_overload_window_s=5.0,
                  overload_rate=100, pool=8, budget=150 * 10**9, tuning=(gr.LAYOUT_BVH2, 128, 12, 0),
                  age_cap_s=2.0, max_wait_s=0.5, log=None):
    """The serving configuration as specified: Poisson arrivals swept over
    `rates` per second, `window_s` seconds of arrivals each, requests drawn from
    the batch configuration's scene, resolution and spp distribution over a
    pool of resident scenes, under an HBM budget. Three server policies:
      fifo       first come first served, every request accepted;
      srf        shortest remaining work first, with an age cap;
      srf_shed   srf plus load shedding: a request the server cannot start
                 within max_wait_s at its measured throughput is refused.
    Without shedding a rate above the server's capacity grows the queue for as
    long as arrivals last, so fifo and srf run their overload rates
    (> overload_rate) for fifo_overload_window_s only; their p99 there is the
    queue's growth over that window."""
    descs = [sc.batch_job(i)[0] for i in range(pool)]
    scenes = [gr.Scene(ctx, d) for d in descs]
    r = np.random.default_rng(0x5EED0005)
    out = {"scene_pool": pool, "budget_bytes": budget, "window_s": window_s,
           "fifo_overload_window_s": fifo_overload_window_s, "age_cap_s": age_cap_s, "max_wait_s": max_wait_s,
           "tuning": {"layout": gr.LAYOUT_NAMES[tuning[0]], "block": tuning[1], "short_stack": tuning[2],
                      "wave_paths": tuning[3] or (1 << 22)}, "runs": []}

    def make_requests(n):
        reqs = []
        for k in range(n):
            si = int(r.integers(0, pool))
            res = int(r.choice(sc.RESOLUTIONS))
            spp = int(r.choice(sc.SPPS))
            reqs.append((si, dict(descs[si].camera, width=res, height=res), spp, k))
        return reqs

    # warm-up: every scene once (graphs captured, pool grown)
    _serve(ctx, scenes, make_requests(2 * pool), budget, 0, 1000.0, tuning)
    for rate in rates:
        for name, policy, cap, wait in (("fifo", gr.SERVER_FIFO, 0.0, 0.0),
                                        ("srf", gr.SERVER_SHORTEST_FIRST, age_cap_s, 0.0),
                                        ("srf_shed", gr.SERVER_SHORTEST_FIRST, age_cap_s, max_wait_s)):
            win = window_s if (wait > 0 or rate <= overload_rate) else fifo_overload_window_s
            reqs = make_requests(max(4, int(rate * win)))
            res = _serve(ctx, scenes, reqs, budget, 0, rate, tuning, policy=policy, age_cap_s=cap, max_wait_s=wait)
            res.update(policy=name, window_s=win)
            out["runs"].append(res)
            if log:
                log("lambda %g %s: %d requests, %d done, %d refused, p50 %.0f ms, p99 %.0f ms, %.1f renders/s, "
                    "%.0f M samples/s" % (rate, name, res["requests"], res["completed"], res["rejected"], res["p50_ms"],
                                          res["p99_ms"], res["renders_s"], res["msamples_s"]))
    for s in scenes:
        s.close()
    return out


def config5(ctx, rates=(10, 20, 50, 100, 200), window_s=3.0, overload_window_s=2.0, overload_rate=50,
            compare_rate=200, compare_requests=150, pool=8, budget=150 * 10**9, tuning=(gr.LAYOUT_BVH2, 128, 12, 0)):
    """Serving sweep; `tuning` = (layout, block, short_stack, wave_paths) of
    the server (tuning_args of an autotuner result). Rates above overload_rate
    (about the server's capacity) run for overload_window_s. The throughput
    comparison — batched server, one job at a time, and the reference's
    per-frame schedule — serves compare_requests requests arriving at
    compare_rate, above every mode's capacity, so renders/s measure capacity,
    not the offered load."""
    descs = [sc.batch_job(i)[0] for i in range(pool)]
    scenes = [gr.Scene(ctx, d) for d in descs]
    r = np.random.default_rng(0x5EED0005)
    layout = tuning[0]
    out = {"scene_pool": pool, "budget_bytes": budget, "window_s": window_s,
           "tuning": {"layout": gr.LAYOUT_NAMES[layout], "block": tuning[1], "short_stack": tuning[2],
                      "wave_paths": tuning[3] or (1 << 22)}, "sweep": []}

    def make_requests(n):
        reqs = []
        for k in range(n):
            si = int(r.integers(0, pool))
            res = int(r.choice(sc.RESOLUTIONS))
            spp = int(r.choice(sc.SPPS))
            cam = dict(descs[si].camera, width=res, height=res)
            reqs.append((si, cam, spp, k))
        return reqs

    for rate in rates:
        reqs = make_requests(max(4, int(rate * (window_s if rate <= overload_rate else overload_window_s))))
        out["sweep"].append(_serve(ctx, scenes, reqs, budget, 0, rate, tuning))
    # the same stream at the highest rate, one job at a time (no batching)
    out["compare_rate"] = compare_rate
    reqs = make_requests(compare_requests)
    out["batched_at_compare_rate"] = _serve(ctx, scenes, reqs, budget, 0, compare_rate, tuning)
    out["sequential_at_compare_rate"] = _serve(ctx, scenes, reqs, budget, 1, compare_rate, tuning)
    out["speedup_renders_s"] = out["batched_at_compare_rate"]["renders_s"] / out["sequential_at_compare_rate"]["renders_s"]
    # the same requests rendered the reference's way, frame by frame, one after
    # another, on scenes created beforehand for each (scene id, resolution)
    views = {}
    for si, cam, _, _ in reqs:
        if (si, cam["width"]) not in views:
            d = descs[si]
            views[(si, cam["width"])] = gr.Scene(ctx, sc.SceneDesc(d.meshes, d.materials, cam, d.env))
            views[(si, cam["width"])].set_tuning(*tuning)
    t = time.perf_counter()
    for si, cam, spp, seed in reqs:
        target = views[(si, cam["width"])]
        target.reset()
        for _ in range(spp):
            target.render(1, 8, seed, flags=gr.RENDER_NO_GRAPH, want_image=False)
    out["per_frame_renders_s"] = len(reqs) / (time.perf_counter() - t)
    for v in views.values():
        v.close()
    out["speedup_vs_per_frame"] = out["batched_at_compare_rate"]["renders_s"] / out["per_frame_renders_s"]
    for s in scenes:
        s.close()
    return out
