"""GPU LBVH build parity: Morton codes, sort order, reference-layout topology,
traversal layout and leaf-order triangles are bit-exact with the oracle and the
reference's golden vectors."""
import os

import numpy as np
import pytest

import gr
import gr.scenes as sc

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "lbvh_ref.npz")


def _cases():
    g = np.load(GOLDEN)
    names = sorted({k.split("/")[0] for k in g.files})
    return [(n, g[n + "/verts"], g[n + "/ref_nodes"], g[n + "/codes"]) for n in names]


def _compare(got, want):
    for k in ("sorted_prim", "sorted_code", "ref_nodes", "nodes", "root"):
        np.testing.assert_array_equal(np.asarray(got[k]), np.asarray(want[k]), err_msg=k)
    np.testing.assert_array_equal(got["tris"].view(np.uint32), want["tris"].view(np.uint32))


@pytest.mark.parametrize("case", _cases(), ids=lambda c: c[0])
def test_gpu_lbvh_matches_reference_golden(ctx, oracle, case):
    name, verts, ref_nodes, codes = case
    b = gr.BVH(ctx)
    b.build_host(verts)
    got = b.export()
    np.testing.assert_array_equal(got["ref_nodes"], ref_nodes)
    np.testing.assert_array_equal(got["sorted_code"], codes[got["sorted_prim"]])
    _compare(got, oracle.lbvh(verts))


# 1,000,000 triangles sort in one cooperative launch (245 tiles of 4,096 keys,
# all resident); 2,000,000 need more tiles than a GB300 holds at once (two per
# SM) and take the four look-back passes.
@pytest.mark.parametrize("n", [2, 3, 4095, 4096, 4097, 65537, 1000000, 2000000])
def test_gpu_lbvh_matches_oracle(ctx, oracle, n):
    v = sc.triangle_soup(n, seed_salt=90 + n % 11)
    if n > 100:
        v[n // 3:n // 3 + 50] = v[n // 3]  # an equal-code run
    b = gr.BVH(ctx)
    b.build_host(v)
    _compare(b.export(), oracle.lbvh(v))


def test_gpu_lbvh_long_equal_run(ctx, oracle):
    # 200,000 triangles with one centroid inside a 1M soup: a 200,000-long run of
    # equal codes, whose gaps find their depth in the run's midpoint subtree
    v = sc.triangle_soup(1000000, seed_salt=96)
    v[300000:500000] = v[300000]
    b = gr.BVH(ctx)
    b.build_host(v)
    _compare(b.export(), oracle.lbvh(v))


def test_gpu_lbvh_all_identical(ctx, oracle):
    v = np.repeat(sc.triangle_soup(1, seed_salt=92), 100000, axis=0)
    b = gr.BVH(ctx)
    b.build_host(v)
    _compare(b.export(), oracle.lbvh(v))


def test_gpu_lbvh_device_input_and_rebuild(ctx, oracle):
    import torch
    v = sc.triangle_soup(200000, seed_salt=93)
    d = torch.from_numpy(v).cuda()
    b = gr.BVH(ctx)
    b.build_device(d, v.shape[0])
    torch.cuda.synchronize()
    first = b.export()
    _compare(first, oracle.lbvh(v))
    # rebuilding in place over a smaller soup reuses the buffers
    v2 = sc.triangle_soup(777, seed_salt=94)
    b.build_host(v2)
    _compare(b.export(), oracle.lbvh(v2))


def test_gpu_lbvh_empty(ctx):
    b = gr.BVH(ctx)
    b.build_host(np.zeros((0, 9), np.float32))
    assert b.export()["root"] == 0xFFFFFFFF


@pytest.mark.parametrize("polls", [1, 1000, 1 << 16])
def test_bounded_wait_gives_up_and_context_stays_usable(ctx, oracle, polls):
    # the build's look-back wait on a status word that nothing publishes and its
    # grid barrier waiting for a block that does not exist: both give up after
    # their poll limit, the call reports GR_ERR_TIMEOUT with the device bit, and
    # the same context then builds and traces as before
    st, bits = ctx.bounded_wait(polls)
    assert st == 5 and bits == 1
    v = sc.triangle_soup(5000, seed_salt=95)
    b = gr.BVH(ctx)
    b.build_host(v)
    _compare(b.export(), oracle.lbvh(v))
