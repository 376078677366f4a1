"""The CPU oracle's LBVH restatement against the reference's own LBVH_build
(golden vectors made by tests/golden/make_golden.py, and the live reference
build in oracle/_ref where it exists)."""
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "lbvh_ref.npz")


def golden_cases():
    g = np.load(GOLDEN)
    names = sorted({k.split("/")[0] for k in g.files})
    return [(n, g[n + "/verts"], g[n + "/ref_nodes"], g[n + "/codes"]) for n in names]


@pytest.mark.parametrize("case", golden_cases(), ids=lambda c: c[0])
def test_oracle_matches_reference_golden(oracle, case):
    name, verts, ref_nodes, codes = case
    got_codes, _ = oracle.morton(verts)
    np.testing.assert_array_equal(got_codes, codes)
    out = oracle.lbvh(verts)
    np.testing.assert_array_equal(out["ref_nodes"], ref_nodes)
    # the sorted order is the leaf sequence of the DFS-preorder node array
    rn = ref_nodes.reshape(-1, 8)
    leaves = rn[rn[:, 7] == 1, 6]
    np.testing.assert_array_equal(out["sorted_prim"], leaves)
    np.testing.assert_array_equal(out["sorted_code"], codes[leaves])


def test_oracle_sorted_order_is_stable(oracle):
    import gr.scenes as sc
    v = sc.triangle_soup(5000, seed_salt=40)
    v[100:300] = v[100]
    out = oracle.lbvh(v)
    c = out["sorted_code"]
    p = out["sorted_prim"]
    assert np.all(np.diff(c.astype(np.int64)) >= 0)
    same = np.diff(c.astype(np.int64)) == 0
    assert np.all(np.diff(p.astype(np.int64))[same] > 0)


@pytest.mark.parametrize("n", [3, 257, 20000, 1000000])
def test_oracle_matches_live_reference(oracle, n):
    if not oracle.ref_available():
        pytest.skip("reference build (oracle/_ref) not present")
    import gr.scenes as sc
    v = sc.triangle_soup(n, seed_salt=50 + n % 7)
    nodes, codes = oracle.ref_lbvh(v)
    got_codes, _ = oracle.morton(v)
    np.testing.assert_array_equal(got_codes, codes)
    np.testing.assert_array_equal(oracle.lbvh(v)["ref_nodes"], nodes)


def test_bvh2_layout_consistent_with_reference_layout(oracle):
    """The gap-indexed traversal layout describes the same tree as the
    reference layout: every internal node's child boxes are the boxes of its
    children, and leaves appear in sorted order."""
    import gr.scenes as sc
    v = sc.triangle_soup(3000, seed_salt=41)
    out = oracle.lbvh(v)
    nodes = out["nodes"].reshape(-1, 16)
    f = nodes.view(np.float32)
    n = v.shape[0]
    seen_leaves = []
    stack = [out["root"]]
    while stack:
        g = stack.pop()
        c0, c1 = nodes[g, 12].view(np.int32), nodes[g, 13].view(np.int32)
        for slot, c in ((0, c0), (1, c1)):
            if c < 0:
                seen_leaves.append(~int(c))
            else:
                assert nodes[c, 14] == g
                stack.append(int(c))
    assert sorted(seen_leaves) == list(range(n))
    assert nodes[out["root"], 14] == 0xFFFFFFFF
    assert f.shape[0] == n - 1
