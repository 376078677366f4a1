"""GPU traversal parity: closest-hit and any-hit results (t, prim, u, v) are
bit-exact with the oracle's restatement of the same FP32 watertight
traversal, and hit ids agree with the reference's traversal on every ray the
FP64 oracle calls unambiguous."""
import numpy as np
import pytest
import torch

import gr
import gr.scenes as sc

pytestmark = pytest.mark.gpu


def _soup(n, salt, scale=1.0):
    v = sc.triangle_soup(n, seed_salt=salt).reshape(n, 3, 3)
    c = v.mean(axis=1, keepdims=True)
    return np.ascontiguousarray(((v - c) * scale + c).reshape(n, 9), np.float32)


def _bits(h):
    return np.ascontiguousarray(h).view(np.uint32)


@pytest.mark.parametrize("n,scale", [(1, 200.0), (2, 200.0), (7, 100.0), (1000, 20.0), (100000, 3.0)])
def test_gpu_trace_bit_exact_small(ctx, oracle, n, scale):
    v = _soup(n, 100 + n, scale)
    b = gr.BVH(ctx)
    b.build_host(v)
    ob = oracle.lbvh(v)
    rays = sc.incoherent_rays(50000, seed_salt=101)
    np.testing.assert_array_equal(_bits(b.trace_host(rays)), _bits(oracle.trace(ob, rays)))
    s = sc.shadow_rays(50000, seed_salt=102)
    np.testing.assert_array_equal(_bits(b.trace_host(s, any_hit=True)), _bits(oracle.trace(ob, s, any_hit=True)))


def test_gpu_trace_config2_sample(ctx, oracle):
    """1M-triangle config-2 scene: bit-exact on incoherent, shadow and coherent
    samples; hit distances within 1e-5 relative of FP64; hit ids equal to the
    reference traversal on unambiguous rays."""
    v = sc.triangle_soup(1000000)
    b = gr.BVH(ctx)
    b.build_host(v)
    ob = oracle.lbvh(v)
    rays = sc.incoherent_rays(4194304)[::16].copy()
    got = b.trace_host(rays)
    np.testing.assert_array_equal(_bits(got), _bits(oracle.trace(ob, rays)))
    s = sc.shadow_rays(4194304)[::16].copy()
    np.testing.assert_array_equal(_bits(b.trace_host(s, any_hit=True)), _bits(oracle.trace(ob, s, any_hit=True)))
    c = sc.coherent_rays()[::16].copy()
    np.testing.assert_array_equal(_bits(b.trace_host(c)), _bits(oracle.trace(ob, c)))
    # reference semantics on unambiguous rays, FP64 distance
    sub = rays[:65536]
    ref = oracle.trace_ref(ob["ref_nodes"], v, sub)
    pr = ref.view(np.int32)[:, 1]
    t64, amb = oracle.fp64_check(ob["ref_nodes"], v, sub, pr)
    pm = got[:65536].view(np.int32)[:, 1]
    ok = ~amb
    assert ok.mean() > 0.99
    np.testing.assert_array_equal(pm[ok], pr[ok])
    hit = ok & (pm >= 0)
    rel = np.abs(got[:65536][hit, 0] - t64[hit]) / np.abs(t64[hit])
    assert rel.max() < 1e-5


def test_gpu_trace_device_pointers_match_host_path(ctx):
    import torch
    v = sc.triangle_soup(300000, seed_salt=103)
    b = gr.BVH(ctx)
    b.build_host(v)
    rays = sc.incoherent_rays(1 << 20, seed_salt=104)
    dr = torch.from_numpy(rays).cuda()
    dh = torch.empty((rays.shape[0], 4), dtype=torch.float32, device="cuda")
    b.trace_device(dr, rays.shape[0], dh, stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(_bits(dh.cpu().numpy()), _bits(b.trace_host(rays)))


def test_gpu_trace_empty_bvh_misses(ctx):
    b = gr.BVH(ctx)
    b.build_host(np.zeros((0, 9), np.float32))
    h = b.trace_host(sc.incoherent_rays(1000, seed_salt=105))
    assert np.all(h.view(np.int32)[:, 1] == -1)


def test_gpu_trace_shared_edge_watertight(ctx):
    q = np.array([[0, 0, 0, 1, 0, 0, 1, 1, 0], [0, 0, 0, 1, 1, 0, 0, 1, 0]], np.float32)
    b = gr.BVH(ctx)
    b.build_host(q)
    t = np.linspace(0.001, 0.999, 4001, dtype=np.float32)
    rays = np.zeros((t.size, 8), np.float32)
    rays[:, 0] = t
    rays[:, 1] = t
    rays[:, 2] = 1.0
    rays[:, 5] = -1.0
    rays[:, 7] = 1e34
    h = b.trace_host(rays)
    assert np.all(h.view(np.int32)[:, 1] == 0)


@pytest.mark.parametrize("any_hit", [False, True])
def test_host_paths_equal_device_path(ctx, any_hit):
    """gr_trace_host with page-locked buffers (traversal reads and writes host
    memory directly) and with pageable buffers (staged in 1 Mi-ray chunks on
    two streams) returns the device path's hits bit for bit."""
    v = sc.triangle_soup(200000, seed_salt=610)
    b = gr.BVH(ctx)
    b.build_host(v)
    b.set_layout(gr.LAYOUT_BVH8_Q8)
    n = (5 << 20) // 2  # 2.5 Mi rays: three chunks when staged
    rays = sc.shadow_rays(n, seed_salt=611) if any_hit else sc.incoherent_rays(n, seed_salt=611)
    dr = torch.from_numpy(rays).cuda()
    dh = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    b.trace_device(dr, n, dh, any_hit=any_hit, stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    want = dh.cpu().numpy().view(np.uint32)
    np.testing.assert_array_equal(b.trace_host(rays, any_hit=any_hit).view(np.uint32), want)  # pageable: staged
    hr = torch.from_numpy(rays).pin_memory()
    hh = torch.zeros((n, 4), dtype=torch.float32).pin_memory()
    ctx.check(gr.load().gr_trace_host(b.h, gr._P(hr.data_ptr()), n, gr._P(hh.data_ptr()), int(any_hit)))
    np.testing.assert_array_equal(hh.numpy().view(np.uint32), want)  # page-locked: direct
