"""The allocation-free LBVH build (gr_bvh_build_noalloc), called through the C
ABI, gives the same BVH as gr_bvh_build, and as the oracle, on two calls in a
row.

It serves callers that cannot call cudaMalloc (plug-ins whose host application
owns all device memory, loops that must not synchronise the device): its
scratch is a fixed array inside the library, so these tests also check that a
second call does not see the first call's leftovers, and that an oversized
request is refused. This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest

import gr
import gr.scenes as sc

pytestmark = pytest.mark.gpu
_P = ctypes.c_void_p
LIMIT = 131072


def _lib():
    L = gr.load()
    f = L.gr_bvh_build_noalloc
    f.argtypes = [_P, _P, ctypes.c_uint32, _P, _P, _P, _P, _P, _P]
    f.restype = ctypes.c_int
    return L


def _build_noalloc(ctx, verts):
    import torch
    n = verts.shape[0]
    d_verts = torch.from_numpy(verts).cuda()
    nodes = torch.full((max(n - 1, 1) * 16,), -7, dtype=torch.int32, device="cuda")
    tris = torch.full((12 * n,), -7.0, dtype=torch.float32, device="cuda")
    prim = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    code = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    header = torch.full((16,), -7, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    st = _lib().gr_bvh_build_noalloc(ctx.h, _P(d_verts.data_ptr()), n, _P(nodes.data_ptr()), _P(tris.data_ptr()),
                                     _P(prim.data_ptr()), _P(code.data_ptr()), _P(header.data_ptr()), _P(stream))
    ctx.check(st, "gr_bvh_build_noalloc")
    torch.cuda.synchronize()
    h = header.cpu().numpy().view(np.uint32)
    return {"nodes": nodes.cpu().numpy().view(np.uint32), "tris": tris.cpu().numpy().view(np.uint32),
            "sorted_prim": prim.cpu().numpy().view(np.uint32), "sorted_code": code.cpu().numpy().view(np.uint32),
            "root": int(h[0]), "err": int(h[2])}


def test_noalloc_build_matches_gr_bvh_build_two_calls(ctx, oracle):
    # a full-size call, then a smaller one over the same fixed scratch
    for n, salt in ((LIMIT, 301), (5000, 302)):
        v = sc.triangle_soup(n, seed_salt=salt)
        v[n // 2:n // 2 + 40] = v[n // 2]  # an equal-code run
        got = _build_noalloc(ctx, v)
        b = gr.BVH(ctx)
        b.build_host(v)
        want = b.export()
        assert got["err"] == 0
        assert got["root"] == want["root"]
        for k in ("sorted_prim", "sorted_code", "nodes"):
            np.testing.assert_array_equal(got[k], want[k], err_msg=k)
        np.testing.assert_array_equal(got["tris"], want["tris"].view(np.uint32))
        b.close()
        # and the oracle's restatement of the reference's LBVH, word for word
        ref = oracle.lbvh(v)
        assert got["root"] == ref["root"]
        for k in ("sorted_prim", "sorted_code", "nodes"):
            np.testing.assert_array_equal(got[k], ref[k], err_msg="oracle " + k)
        np.testing.assert_array_equal(got["tris"], ref["tris"].view(np.uint32))


def test_noalloc_build_refuses_oversize(ctx):
    L = _lib()
    st = L.gr_bvh_build_noalloc(ctx.h, None, LIMIT + 1, None, None, None, None, None, None)
    assert st == 1  # GR_ERR_INVALID
    assert b"131072" in L.gr_last_error(ctx.h)
