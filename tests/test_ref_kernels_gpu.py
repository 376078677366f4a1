"""The reference's own traversal kernels on the GPU.

`trace_kernel` and `trace_shadow_kernel` (pathtracer_kernel.h:175-321) are
compiled from the reference sources (oracle/ref/build_ref.sh) and launched as
the reference launches them (oracle/ref_gpu.py). They pin two things:

* the CPU restatement of the reference traversal (oracle/trace.cpp
  `or_trace_ref`): with --fmad=false the kernels round every float operation
  as written, as the restatement does, and the two agree bit for bit — triangle
  id on every ray, t / u / v on every hit, closest and any hit;
* our traversal against the reference as shipped (nvcc's default flags, FMA
  contraction on): hit ids equal on every ray that is not ambiguous in FP64
  (another hit within 1e-6 relative, or the hit within 1e-6 of an edge, as a
  barycentric or in world units relative to the coordinates' magnitude),
  distances within 1e-5 relative of FP64 plus the FP32 rounding of the
  triangle's plane along the ray.
"""
import numpy as np
import pytest
import torch

import gr
import gr.scenes as sc
import ref_gpu

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not (ref_gpu.available("stock") and ref_gpu.available("nofma")),
                                 reason="reference kernels not built (reference sources absent at build time)")]


@pytest.fixture(scope="module")
def nofma():
    rk = ref_gpu.RefKernels("nofma")
    yield rk
    rk.close()


@pytest.fixture(scope="module")
def stock():
    rk = ref_gpu.RefKernels("stock")
    yield rk
    rk.close()


def _soup(n, salt, scale=1.0):
    v = sc.triangle_soup(n, seed_salt=salt).reshape(n, 3, 3)
    c = v.mean(axis=1, keepdims=True)
    return np.ascontiguousarray(((v - c) * scale + c).reshape(n, 9), np.float32)


def _ids(h):
    return np.ascontiguousarray(h).view(np.int32)[:, 1]


def _assert_same_records(got, want):
    """Triangle id on every ray; t, u, v bits on hits (a miss leaves them unset
    in the reference kernels)."""
    gi, wi = _ids(got), _ids(want)
    np.testing.assert_array_equal(gi, wi)
    hit = wi >= 0
    gb = np.ascontiguousarray(got).view(np.uint32)[hit]
    wb = np.ascontiguousarray(want).view(np.uint32)[hit]
    np.testing.assert_array_equal(gb[:, [0, 2, 3]], wb[:, [0, 2, 3]])


@pytest.mark.parametrize("n,scale", [(1, 200.0), (2, 200.0), (7, 100.0), (1000, 20.0), (100000, 3.0)])
def test_restatement_equals_reference_kernels(oracle, nofma, n, scale):
    v = _soup(n, 300 + n, scale)
    nodes = oracle.lbvh(v)["ref_nodes"]
    scene = nofma.scene(nodes, v)
    rays = sc.incoherent_rays(50000, seed_salt=301)
    got = nofma.trace_host(scene, rays)
    want = oracle.trace_ref(nodes, v, rays)
    assert (_ids(want) >= 0).any()
    _assert_same_records(got, want)
    s = sc.shadow_rays(50000, seed_salt=302)
    _assert_same_records(nofma.trace_host(scene, s, any_hit=True), oracle.trace_ref(nodes, v, s, any_hit=True))


def test_restatement_equals_reference_kernels_config2(ctx, oracle, nofma):
    """The full workload: 1M-triangle tree built by our GPU LBVH (the reference
    topology), all 4,194,304 incoherent rays, 4,194,304 shadow rays and the
    2048x2048 coherent grid."""
    v = sc.triangle_soup(1000000)
    b = gr.BVH(ctx)
    b.build_host(v)
    nodes = b.export()["ref_nodes"]
    scene = nofma.scene(nodes, v)
    rays = sc.incoherent_rays(4194304)
    _assert_same_records(nofma.trace_host(scene, rays), oracle.trace_ref(nodes, v, rays))
    s = sc.shadow_rays(4194304)
    _assert_same_records(nofma.trace_host(scene, s, any_hit=True), oracle.trace_ref(nodes, v, s, any_hit=True))
    c = sc.coherent_rays()
    _assert_same_records(nofma.trace_host(scene, c), oracle.trace_ref(nodes, v, c))


def test_gr_agrees_with_reference_as_shipped_config2(ctx, oracle, stock):
    """All 4,194,304 incoherent rays of the workload: every ray on which our
    closest hit and the shipped reference kernel's differ is ambiguous in FP64;
    on the others both distances agree with FP64."""
    v = sc.triangle_soup(1000000)
    b = gr.BVH(ctx)
    b.build_host(v)
    nodes = b.export()["ref_nodes"]
    scene = stock.scene(nodes, v)
    rays = sc.incoherent_rays(4194304)
    dr = torch.from_numpy(rays).cuda()
    ref = torch.zeros((rays.shape[0], 4), dtype=torch.float32, device="cuda")
    mine = torch.zeros_like(ref)
    stock.trace(scene, dr, ref)
    b.trace_device(dr, rays.shape[0], mine, stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    ref, mine = ref.cpu().numpy(), mine.cpu().numpy()
    pr, pm = _ids(ref), _ids(mine)
    assert (pr >= 0).mean() > 0.3
    diff = np.nonzero(pr != pm)[0]
    assert diff.size < rays.shape[0] * 1e-3
    if diff.size:
        _, amb = oracle.fp64_check(nodes, v, rays[diff], pr[diff])
        assert amb.all(), "%d of %d differing rays are not ambiguous: %s" % ((~amb).sum(), diff.size, diff[~amb][:10])
        # the first ambiguity definition (another hit within 1e-6 relative, or a
        # barycentric within 1e-6 of an edge), without the world-unit edge
        # criterion: the rays it does not call ambiguous are few, and each is
        # ambiguous under the FP32 resolution of its coordinates
        _, amb_rel = oracle.fp64_check(nodes, v, rays[diff], pr[diff], edge_rel=0.0)
        print("differing rays: %d of %d; ambiguous under the relative criteria alone: %d; with the world-unit "
              "edge criterion: %d" % (diff.size, rays.shape[0], int(amb_rel.sum()), int(amb.sum())))
        assert (~amb_rel).sum() <= 64
    # distances on every 16th common hit against FP64: within 1e-5 relative
    # (1e-8 absolute below t = 1e-3) plus the FP32 rounding of the plane
    # position along the ray, 1e-7 / |cos| (ray direction against the normal)
    hit = np.nonzero((pr == pm) & (pr >= 0))[0][::16]
    t64, amb = oracle.fp64_check(nodes, v, rays[hit], pr[hit])
    ok = hit[~amb]
    t64 = t64[~amb]
    p = v[pr[ok]].reshape(-1, 3, 3).astype(np.float64)
    d = rays[ok, 3:6].astype(np.float64)
    nrm = np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0])
    cos = np.abs((d * nrm).sum(1)) / np.linalg.norm(d, axis=1) / np.linalg.norm(nrm, axis=1)
    scale = 1e-5 * np.maximum(np.abs(t64), 1e-3)
    assert np.all(np.abs(mine[ok, 0] - t64) <= scale + 1e-7 / cos)
    # the reference's mixed-precision Moller-Trumbore loses more near grazing
    # incidence; it is held to a looser plane term
    assert np.all(np.abs(ref[ok, 0] - t64) <= scale + 1e-6 / cos)


def test_reference_shadow_kernel_agrees_on_occlusion(ctx, stock):
    """Any hit: occluded or not, per ray, equal between our traversal and the
    shipped reference kernel on shadow rays (the triangle reported may differ:
    both stop at the first accepted hit, in different visit orders)."""
    v = sc.triangle_soup(1000000)
    b = gr.BVH(ctx)
    b.build_host(v)
    scene = stock.scene(b.export()["ref_nodes"], v)
    s = sc.shadow_rays(1 << 20, seed_salt=303)
    got = b.trace_host(s, any_hit=True)
    ref = stock.trace_host(scene, s, any_hit=True)
    occ_g, occ_r = _ids(got) >= 0, _ids(ref) >= 0
    assert occ_r.mean() > 0.05
    assert (occ_g != occ_r).mean() < 1e-4
