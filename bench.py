#!/usr/bin/env python3
"""Benchmark of the wavefront render path's traversal on the LBVH microbench
workload: 1,000,000 triangles (centroids uniform in the unit cube, lognormal
edges), 4,194,304 incoherent rays (origins uniform in the cube, directions
uniform on the sphere), closest-hit queries, FP32, 30-bit Morton LBVH.

One step = one closest-hit pass over the 4M rays with rays and BVH resident in
HBM. The L2 is flushed (a 256 MB write) before every timed step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gr|reference]

Prints one JSON line (rank 0). `--impl reference` times the reference's
traversal semantics (pathtracer_kernel.h:175-233, restated on the CPU because
the reference has no CPU traversal) on the host cores, on a bounded sample.
Both lines also carry `reference_gpu`: the reference's own kernels, compiled
from its sources for sm_103a, timed on the GPU — its traversal kernels on the
same tree and rays, and its whole frame loop on the Cornell-box and glossy
render configurations (when those kernels were built).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "gpu-renderer_gb300"))

import numpy as np  # noqa: E402

N_TRIS = 1_000_000
N_RAYS = 4_194_304
METRIC = "incoherent closest-hit Mrays/s (1M-triangle LBVH, 4M rays)"
UNIT = "Mrays/s"
WORKLOAD = "lbvh-traversal-microbench: 1M tris, 4M incoherent rays, closest hit"
# Algorithmic bytes per ray, from the reference traversal's node/triangle visit
# counts on this ray set (CPU oracle, 262,144-ray sample): V_node = 348.44,
# V_tri = 4.63; B_ray = 32 (ray) + 16 (hit) + 32 V_node + 36 V_tri.
V_NODE_REF = 348.44
V_TRI_REF = 4.63
BYTES_PER_RAY = 32 + 16 + 32 * V_NODE_REF + 36 * V_TRI_REF
FALLBACK_HBM_GBS = 6800.0


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle samples taken while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, ValueError):
            self.proc = None
            return
        # nvidia-smi's start-up (NVML initialisation) stalled the next CUDA
        # launch by about 0.9 s on GB300: the timed region opens only after the
        # first sample has arrived
        deadline = time.perf_counter() + 5.0
        while not self.lines and self.proc.poll() is None and time.perf_counter() < deadline:
            time.sleep(0.01)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def cpu_reference(steps, warmup, sample_rays=262144):
    """The reference traversal (closest hit, right-first, FP64 Moller-Trumbore)
    restated on the CPU, all host threads, on a bounded sample of the rays."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    from gr import scenes
    verts = scenes.triangle_soup(N_TRIS)
    rays = scenes.incoherent_rays(N_RAYS)
    stride = max(1, N_RAYS // sample_rays)
    sample = np.ascontiguousarray(rays[::stride][:sample_rays])
    bvh = pyoracle.lbvh(verts)
    threads = pyoracle.threads()
    for _ in range(warmup):
        pyoracle.trace_ref(bvh["ref_nodes"], verts, sample[:4096], nthreads=threads)
    times = []
    st = None
    for _ in range(steps):
        t0 = time.perf_counter()
        _, st = pyoracle.trace_ref(bvh["ref_nodes"], verts, sample, stats=True, nthreads=threads)
        times.append(time.perf_counter() - t0)
    value = sample.shape[0] * len(times) / sum(times) / 1e6
    return {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "%d of the %d incoherent rays (every %dth), reference traversal semantics "
                      "(pathtracer_kernel.h:175-233) restated in C++, %d threads" % (
                          sample.shape[0], N_RAYS, stride, threads),
            "v_node": float(st[:, 0].mean()), "v_tri": float(st[:, 1].mean()),
            "seconds_per_step": sum(times) / len(times)}


def reference_gpu(verts, ref_nodes, rays_by_query, flush, steps):
    """The reference's own trace_kernel / trace_shadow_kernel
    (pathtracer_kernel.h:175-321), compiled from its sources for sm_103a with
    nvcc's default flags and launched as its trace() wrappers do, timed on the
    same triangles, tree topology and rays as ours (CUDA events, L2 flushed
    before every launch). None when the kernels were not built."""
    import torch
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ref_gpu
    if not ref_gpu.available("stock"):
        return {"unavailable": "reference kernels not built (the reference sources were absent at build time)"}
    rk = ref_gpu.RefKernels("stock")
    try:
        scene = rk.scene(ref_nodes, verts)
        stream = torch.cuda.current_stream()
        out = {"kernel": "trace_kernel / trace_shadow_kernel (pathtracer_kernel.h:175-321)",
               "build": "reference sources, nvcc defaults (device -O3, FMA contraction on), sm_103a cubin",
               "launch": "32-thread blocks, one ray per thread (pathtracer_kernel.h:235-246, 310-321)",
               "tree": "reference LBVH topology (equal to LBVH_build word for word), depth %d" % scene.depth}
        for name, (d_rays, any_hit) in rays_by_query.items():
            m = d_rays.shape[0]
            d_hits = torch.empty((m, 4), dtype=torch.float32, device=d_rays.device)
            for _ in range(3):
                rk.trace(scene, d_rays, d_hits, any_hit)
            ms = []
            for _ in range(max(3, min(steps, 10))):
                l2_flush(flush)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                rk.trace(scene, d_rays, d_hits, any_hit)
                e1.record(stream)
                torch.cuda.synchronize()
                ms.append(e0.elapsed_time(e1))
            out[name + "_mrays_s"] = m / (statistics.median(ms) / 1e3) / 1e6
            del d_hits
        del scene
        return out
    finally:
        rk.close()


def reference_gpu_renders(nodes_for):
    """The reference's whole frame loop on the GPU — its own kernels (compiled
    from its sources, nvcc defaults) over the scene records its loader builds,
    driven as PathTracer::render(uint32*) drives them (pathtracer.cu:41-150, a
    device synchronise after every kernel) — for the Cornell box (256x256, 16
    frames, depth 8) and the glossy scene (1024x768, 64 frames, depth 16), and
    the 64 jobs of the batched configuration one after another (each job's spp
    as frames, depth 8). `nodes_for(desc)` gives the reference-layout tree of
    the scene's soup. Wall-clock time of the frames (after one warm-up frame
    for the two single scenes); building the records is not timed."""
    import torch
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ref_gpu
    from gr import scenes
    if not ref_gpu.render_available("stock"):
        return {"unavailable": "reference kernels or frame driver not built"}
    rk = ref_gpu.RefKernels("stock")
    out = {}
    try:
        for name, make, spp, depth in (("config1_render", lambda: scenes.cornell_box(256, 256), 16, 8),
                                       ("config3_render", scenes.glossy_scene, 64, 16)):
            desc = make()
            rr = ref_gpu.RefRender(rk, desc, nodes_for(desc))
            rr.render(1, depth)
            secs, rays = rr.render(spp, depth)
            npix = rr.width * rr.height
            out[name] = {"ms": secs * 1e3, "samples_per_s": npix * spp / secs, "mrays_s": rays / secs / 1e6,
                         "frames": spp, "max_path_length": depth, "triangles": rr.triangles}
            del rr, desc
            torch.cuda.empty_cache()
        # the 64-job stream of the batched configuration, one reference render
        # per job (depth 8), as the reference renders scenes one after another
        total, samples, setup = 0.0, 0, 0.0
        n_jobs = 64
        for i in range(n_jobs):
            desc, spp = scenes.batch_job(i)
            t0 = time.perf_counter()
            rr = ref_gpu.RefRender(rk, desc, nodes_for(desc))
            setup += time.perf_counter() - t0
            secs, _ = rr.render(spp, 8)
            total += secs
            samples += rr.width * rr.height * spp
            del rr, desc
            torch.cuda.empty_cache()
        out["config4_sequential"] = {"jobs": n_jobs, "renders_s": n_jobs / total, "seconds": total,
                                     "samples_per_s": samples / total, "setup_seconds_excluded": setup}
    finally:
        rk.close()
    out["timing"] = "wall clock of the frame loop, which synchronises the device after every kernel as the reference does"
    return out


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    cb = cpu_reference(max(args.steps, 1), max(args.warmup, 0) and 1)
    rg = None
    if not args.no_reference_gpu:
        import torch
        if torch.cuda.is_available():
            from gr import scenes
            sys.path.insert(0, os.path.join(ROOT, "oracle"))
            import pyoracle
            verts = scenes.triangle_soup(N_TRIS)
            dev = torch.device("cuda", 0)
            torch.cuda.set_device(0)
            flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
            queries = {"closest": (torch.from_numpy(scenes.incoherent_rays(N_RAYS)).to(dev), False),
                       "coherent_closest": (torch.from_numpy(scenes.coherent_rays()).to(dev), False),
                       "shadow_anyhit": (torch.from_numpy(scenes.shadow_rays(N_RAYS)).to(dev), True)}
            rg = reference_gpu(verts, pyoracle.lbvh(verts)["ref_nodes"], queries, flush, args.steps)
            del queries, flush
            if "unavailable" not in rg:
                rg.update(reference_gpu_renders(lambda desc: pyoracle.lbvh(desc.flatten()[0])["ref_nodes"]))
    out = {
        "impl": "reference", "metric": METRIC, "value": cb["value"], "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": cb["seconds_per_step"] * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "sample": cb["sample"]},
        "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
        "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    if rg is not None:
        out["reference_gpu"] = rg
    print(json.dumps(out), flush=True)


def whole_job(local_seconds, units_per_rank, device):
    """Replicas (one process per GPU, no exchange on the data path): the job
    takes as long as its slowest rank, and its work is the units of all ranks.
    Returns (million units per second over the whole job, max seconds)."""
    import torch
    import torch.distributed as dist
    ws = dist.get_world_size() if dist.is_available() and dist.is_initialized() else 1
    t = float(local_seconds)
    if ws > 1:
        x = torch.tensor([t], device=device, dtype=torch.float64)
        dist.all_reduce(x, op=dist.ReduceOp.MAX)
        t = float(x.item())
    return ws * units_per_rank / t / 1e6, t


# LBVH build, algorithmic bytes per triangle: 36 vertex read for the Morton
# codes, 8 code / index write, 4 sort passes x 16, 36 vertex re-read for the
# leaf boxes, 2 x 32 node writes, 8 parent links and counters.
BUILD_BYTES_PER_TRI = 216


def _binding(entry, event_ms, peak):
    """What binds a kernel, from its committed ncu figures: DRAM bytes per
    launch over the event-timed duration against the HBM peak, the L2 and
    issue figures of the smaller capture of the same kernel."""
    full, small = entry["full"], entry["small"]
    traffic = full["dram_bytes_read"] + full["dram_bytes_write"]
    dram_gbs = traffic / (event_ms / 1e3) / 1e9
    return {"resource": "instruction issue",
            "issue_active": small["issue_active_pct"] / 100,
            "threads_per_warp_instruction": small["threads_per_warp_instruction"],
            "dram_gbs": dram_gbs, "dram_frac_of_peak": dram_gbs / peak,
            "l2_frac_of_peak": small["l2_throughput_pct_of_peak"] / 100,
            "l2_hit_rate": small["l2_hit_rate_pct"] / 100,
            "l2_bytes_per_ray": small["lts_bytes"] / small["rays"],
            "warp_instructions_per_ray": small["warp_instructions"] / small["rays"],
            "captured_rays": [full["rays"], small["rays"]]}, traffic


def roofline_block(layout_name, achieved, peak, peak_kind, closest_ms, anyhit_ms, build_ms):
    """The roofline entry of the JSON line. It leads with what binds the
    headline kernel (measured: instruction issue at about half the lanes of a
    warp, with DRAM and L2 far from their peaks), then gives the contract's
    algorithmic-byte figure, whose bytes are the reference traversal's (its
    348 node visits per ray on its binary tree): a fraction above 1 means L2
    reuse and fewer visits, not HBM traffic. Any-hit and the LBVH build get
    the same treatment."""
    path = os.path.join(ROOT, "profiles", "roofline_inputs.json")
    inputs = {}
    if os.path.exists(path):
        with open(path) as f:
            inputs = json.load(f)
    out = {}
    traffic = None
    captured = layout_name == "bvh8_q8"  # the captures are of the 8-wide kernels
    if captured and "closest" in inputs:
        out["binding"], traffic = _binding(inputs["closest"], closest_ms, peak)
    out.update({"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "peak_kind": peak_kind, "traffic": traffic,
                "kernel": "k_trace<closest, %s>" % layout_name, "bytes_per_ray": BYTES_PER_RAY,
                "achieved_is": "reference-traversal bytes (11,364.8 B/ray: the reference's node and triangle "
                               "fetches on its binary tree) per event-timed launch; above 1 of HBM = L2 reuse and "
                               "fewer node visits, not DRAM traffic (see binding)"})
    if captured and "anyhit" in inputs and anyhit_ms:
        b, t = _binding(inputs["anyhit"], anyhit_ms, peak)
        out["anyhit"] = {"kernel": "k_trace<any hit, %s>" % layout_name, "kernel_ms": anyhit_ms,
                         "traffic": t, "binding": b}
    if "build" in inputs and build_ms:
        b = inputs["build"]
        alg = BUILD_BYTES_PER_TRI * b["triangles"]
        t = b["dram_bytes_read"] + b["dram_bytes_write"]
        out["build"] = {"kernel": "LBVH build (%d launches), %d triangles" % (b["launches"], b["triangles"]),
                        "ms": build_ms,
                        "achieved": alg / (build_ms / 1e3) / 1e9, "frac": alg / (build_ms / 1e3) / 1e9 / peak,
                        "unit": "GB/s", "algorithmic_bytes": alg, "traffic": t,
                        "dram_frac_of_peak": t / (build_ms / 1e3) / 1e9 / peak,
                        "binding": "latency: dependent launches, the sort's look-back and the bottom-up "
                                   "climbs (longest: %s)" % ", ".join("%s %.0f us" % (k, v / 1e3)
                                                             for k, v in b["longest"].items())}
    return out


def l2_flush(buf):
    buf.zero_()


def run_gpu(args):
    import torch
    import gr
    from gr import scenes

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    n_tris, n_rays = args.tris, args.rays
    verts = scenes.triangle_soup(n_tris)
    # --quick --any-hit times the shadow any-hit query instead (profiling)
    quick_any = bool(args.quick and args.any_hit)
    rays = scenes.shadow_rays(n_rays) if quick_any else scenes.incoherent_rays(n_rays)
    ctx = gr.Context(local)
    bvh = gr.BVH(ctx)
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    d_verts = torch.from_numpy(verts).to(dev)
    d_rays = torch.from_numpy(rays).to(dev)
    d_hits = torch.empty((max(n_rays, N_RAYS), 4), dtype=torch.float32, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    # BVH build (timed separately, reported as an extra)
    build_ms = []
    for i in range(3 + 5):
        l2_flush(flush)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        bvh.build_device(d_verts, n_tris, stream=sp)
        e1.record(stream)
        torch.cuda.synchronize()
        if i >= 3:
            build_ms.append(e0.elapsed_time(e1))
    # the 8-wide 8-bit layout collapsed from a fresh build (wall clock: the
    # collapse reads each level's size back to the host)
    collapse_ms = []
    for i in range(3 + 3):
        bvh.set_layout(gr.LAYOUT_BVH2, stream=sp)  # a rebuild keeps the current layout built
        bvh.build_device(d_verts, n_tris, stream=sp)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        bvh.set_layout(gr.LAYOUT_BVH8_Q8, stream=sp)
        torch.cuda.synchronize()
        if i >= 3:
            collapse_ms.append((time.perf_counter() - t0) * 1e3)

    def step(buf_rays, buf_hits, n, any_hit=False):
        bvh.trace_device(buf_rays, n, buf_hits, any_hit=any_hit, stream=sp)

    # traversal configuration: the autotuner times every node layout x block
    # x short-stack configuration on the workload's rays (untimed for the
    # result) and keeps the fastest; all of them return the same hits
    names = {v: k for k, v in gr.LAYOUT_NAMES.items()}
    torch.cuda.synchronize()
    if args.layout == "auto":
        table = bvh.autotune(d_rays, n_rays, d_hits, any_hit=quick_any)
    else:
        bvh.set_tuning(names[args.layout], args.block, args.short_stack)
        table = []
    torch.cuda.synchronize()
    tuning = bvh.tuning()
    layout = names[tuning["layout"]]
    layout_rates = {"%s/%d/%d" % (t["layout"], t["block"], t["short_stack"]): round(n_rays / ms / 1e3, 1)
                    for t, ms in table}

    for _ in range(max(args.warmup, 3)):
        step(d_rays, d_hits, n_rays, quick_any)
    torch.cuda.synchronize()

    clocks = ClockSampler(local)
    clocks.start()
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    ev = []
    for _ in range(args.steps):
        l2_flush(flush)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step(d_rays, d_hits, n_rays, quick_any)
        e1.record(stream)
        ev.append((e0, e1))
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    kernel_ms = [a.elapsed_time(b) for a, b in ev]
    total_s = sum(kernel_ms) / 1e3

    if args.quick:
        clocks.stop()
        if rank == 0:
            print(json.dumps({"quick": True, "query": "any hit" if quick_any else "closest hit", "tris": n_tris,
                              "rays": n_rays, "tuning": tuning,
                              "autotune_mrays_s": layout_rates,
                              "kernel_ms_median": statistics.median(kernel_ms),
                              "mrays_s": n_rays / (statistics.median(kernel_ms) / 1e3) / 1e6}), flush=True)
        return

    # secondary queries on the same scene: coherent closest hit and shadow any-hit
    extras = {}
    for name, gen, anyh in (("coherent_closest", scenes.coherent_rays, False),
                            ("shadow_anyhit", scenes.shadow_rays, True)):
        r2 = gen() if name == "coherent_closest" else gen(N_RAYS)
        d_r2 = torch.from_numpy(r2).to(dev)
        for _ in range(3):
            step(d_r2, d_hits, r2.shape[0], anyh)
        ms = []
        for _ in range(max(3, min(args.steps, 10))):
            l2_flush(flush)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step(d_r2, d_hits, r2.shape[0], anyh)
            e1.record(stream)
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
        extras[name + "_mrays_s"] = r2.shape[0] / (statistics.median(ms) / 1e3) / 1e6
        extras[name + "_kernel_ms"] = statistics.median(ms)
        del d_r2
    if rank == 0 and not args.no_reference_gpu:
        d_s = torch.from_numpy(scenes.shadow_rays(N_RAYS)).to(dev)
        d_c = torch.from_numpy(scenes.coherent_rays()).to(dev)
        rg = reference_gpu(verts, bvh.export()["ref_nodes"],
                           {"closest": (d_rays, False), "coherent_closest": (d_c, False),
                            "shadow_anyhit": (d_s, True)}, flush, args.steps)
        if "closest_mrays_s" in rg:
            rg["gr_over_reference_closest"] = (n_rays / (statistics.median(kernel_ms) / 1e3) / 1e6) / rg["closest_mrays_s"]
        extras["reference_gpu"] = rg
        del d_s, d_c
    clock_info = clocks.stop()

    # render configurations (plain render, batched, serving)
    if not args.no_render:
        from gr import workloads as wl
        log = lambda m: print("[bench] " + m, file=sys.stderr, flush=True)  # noqa: E731
        log("config 1 (Cornell box 256x256, 16 spp, depth 8)")
        extras["config1_render"] = wl.plain_render(ctx, scenes.cornell_box(256, 256), 16, 8)
        log("config 3 (glossy scene 1024x768, 64 spp, depth 16)")
        extras["config3_render"] = wl.plain_render(ctx, scenes.glossy_scene(), 64, 16)
        log("config 4 (64-job batch, default and autotuned configuration)")
        extras["config4_batch"] = wl.config4(ctx)
        log("config 5 (serving sweep, config 4's autotuned configuration)")
        c4 = extras["config4_batch"].get("autotune")
        tuned = wl.tuning_args(c4["tuning"], c4["wave_paths"]) if c4 else (gr.LAYOUT_BVH2, 128, 12, 0)
        extras["config5_serving"] = wl.config5(ctx, tuning=tuned)
        if rank == 0 and not args.no_reference_gpu and "reference_gpu" in extras:
            log("reference kernels: config 1 and config 3 frame loops")

            def gr_nodes(desc):
                t = gr.BVH(ctx)
                t.build_host(desc.flatten()[0])
                return t.export()["ref_nodes"]

            rr = reference_gpu_renders(gr_nodes)
            for k in ("config1_render", "config3_render"):
                if k in rr and k in extras:
                    rr[k]["gr_speedup"] = rr[k]["ms"] / extras[k]["ms"]
            c4 = extras.get("config4_batch", {}).get("autotuned")
            if "config4_sequential" in rr and c4:
                rr["config4_sequential"]["gr_batched_speedup"] = c4["batched_renders_s"] / rr["config4_sequential"]["renders_s"]
            extras["reference_gpu"].update(rr)

    # end to end through the C ABI with host buffers (pinned), copies inside
    h_rays = torch.from_numpy(rays).pin_memory()
    h_hits = torch.empty((N_RAYS, 4), dtype=torch.float32).pin_memory()
    L = gr.load()
    for _ in range(2):
        ctx.check(L.gr_trace_host(bvh.h, gr._P(h_rays.data_ptr()), N_RAYS, gr._P(h_hits.data_ptr()), 0))
    e2e_t = []
    for _ in range(max(3, min(args.steps, 10))):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx.check(L.gr_trace_host(bvh.h, gr._P(h_rays.data_ptr()), N_RAYS, gr._P(h_hits.data_ptr()), 0))
        e2e_t.append(time.perf_counter() - t0)
    e2e_value = N_RAYS * len(e2e_t) / sum(e2e_t) / 1e6

    # whole-job value: max time over ranks, rays over all ranks
    value, t_max = whole_job(total_s, n_rays * args.steps, dev)

    if rank == 0:
        peak, peak_kind = measured_peaks()
        avg_ms = sum(kernel_ms) / len(kernel_ms)
        achieved = BYTES_PER_RAY * N_RAYS / (avg_ms / 1e3) / 1e9
        build_ms = statistics.median(build_ms)
        roofline = roofline_block(layout_name=gr.LAYOUT_NAMES[layout], achieved=achieved, peak=peak,
                                  peak_kind=peak_kind, closest_ms=avg_ms,
                                  anyhit_ms=extras.get("shadow_anyhit_kernel_ms"), build_ms=build_ms)
        cb = cpu_reference(1, 0)
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_max * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "triangles": N_TRIS, "rays": N_RAYS, "query": "closest hit",
                       "tuning": tuning, "autotune_mrays_s": layout_rates,
                       "l2": "flushed (256 MB write) before every timed step", "parallelism": "replicas"},
            "roofline": roofline,
            "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": N_RAYS * 32,
                    "d2h_bytes_per_step": N_RAYS * 16, "api": "gr_trace_host with page-locked host rays and hits: the traversal reads the rays and "
                           "writes the hits in host memory over the host link inside the timed region"},
            "gpu_launches": args.steps,
            "clocks": clock_info,
            "extra": dict(extras, bvh_build_ms=build_ms,
                          bvh_build_mtris_s=N_TRIS / (build_ms / 1e3) / 1e6,
                          bvh8_collapse_ms=statistics.median(collapse_ms),
                          kernel_ms_median=statistics.median(kernel_ms)),
        }
        print(json.dumps(out), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def run_render_only(args):
    import torch
    import gr
    from gr import scenes
    from gr import workloads as wl

    torch.cuda.set_device(0)
    ctx = gr.Context(0)
    desc, spp, depth = ((scenes.cornell_box(256, 256), 16, 8) if args.render_only == "config1" else
                        (scenes.glossy_scene(), 64, 16))
    names = {v: k for k, v in gr.LAYOUT_NAMES.items()}
    lay = names["bvh2" if args.layout == "auto" else args.layout]
    out = wl.plain_render(ctx, desc, args.spp or spp, depth, autotune=False,
                          tuning=(lay, args.block, args.short_stack, args.wave_paths))
    print(json.dumps(dict(out, workload=args.render_only)), flush=True)


def run_serving_sweep(args):
    """The serving configuration's full sweep (not part of the default run:
    about six minutes): prints one JSON line of per-rate, per-policy latency
    and throughput."""
    import torch
    import gr
    from gr import workloads as wl
    torch.cuda.set_device(0)
    ctx = gr.Context(0)
    names = {v: k for k, v in gr.LAYOUT_NAMES.items()}
    tuning = (names[args.layout if args.layout != "auto" else "bvh8_q8"], args.block, args.short_stack,
              args.wave_paths)
    log = lambda m: print("[serving] " + m, file=sys.stderr, flush=True)  # noqa: E731
    out = wl.config5_sweep(ctx, window_s=args.window, tuning=tuning, log=log)
    print(json.dumps(dict(out, workload="serving sweep (Poisson arrivals, config-4 request distribution)")),
          flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gr", choices=["gr", "reference"])
    ap.add_argument("--tris", type=int, default=N_TRIS, help="triangle count (profiling cases)")
    ap.add_argument("--rays", type=int, default=N_RAYS, help="ray count (profiling cases)")
    ap.add_argument("--no-render", action="store_true", help="skip the render-configuration extras")
    ap.add_argument("--no-reference-gpu", action="store_true",
                    help="skip timing the reference's own traversal kernels on the GPU")
    ap.add_argument("--layout", default="auto", choices=["auto", "bvh2", "bvh4", "bvh4_q8", "bvh8_q8"],
                    help="node layout of the timed traversal (auto: autotune layout, block and short stack)")
    ap.add_argument("--block", type=int, default=128, choices=[64, 128, 256])
    ap.add_argument("--short-stack", type=int, default=12, choices=[8, 12, 16])
    ap.add_argument("--any-hit", action="store_true",
                    help="with --quick: time the shadow any-hit query (profiling the any-hit kernel)")
    ap.add_argument("--quick", action="store_true",
                    help="time the main query only (no extras, e2e or CPU baseline); for profiling")
    ap.add_argument("--render-only", default=None, choices=["config1", "config3"],
                    help="render one configuration with the given --layout/--block/--short-stack and --spp, print "
                         "its figures and exit (profiling the integrator's kernels)")
    ap.add_argument("--spp", type=int, default=0, help="samples per pixel of --render-only (0: the configuration's)")
    ap.add_argument("--wave-paths", type=int, default=0,
                    help="paths per wave of --render-only (0: the library's default)")
    ap.add_argument("--serving-sweep", action="store_true",
                    help="run the serving configuration's full sweep (rates 10-500/s, three server policies) and exit")
    ap.add_argument("--window", type=float, default=20.0, help="seconds of arrivals per rate of --serving-sweep")
    args = ap.parse_args()
    if args.serving_sweep:
        run_serving_sweep(args)
    elif args.render_only:
        run_render_only(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
