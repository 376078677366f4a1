"""Host-side checks of the launcher for the reference's own traversal kernels
(oracle/ref_gpu.py): the tree walk that guards every launch, and the record
layout it reads. No GPU."""
import json
import os

import numpy as np
import pytest

import gr.scenes as sc
import ref_gpu


def _depth_recursive(nodes, i=0):
    w = nodes.reshape(-1, 8)
    if w[i, 7] & 0xFF:
        return 0
    return 1 + max(_depth_recursive(nodes, i + 1), _depth_recursive(nodes, int(w[i, 6])))


@pytest.mark.parametrize("n", [1, 2, 3, 7, 64, 1000])
def test_tree_depth_matches_recursive_walk(oracle, n):
    v = sc.triangle_soup(n, seed_salt=400 + n)
    nodes = oracle.lbvh(v)["ref_nodes"]
    assert ref_gpu.tree_depth(nodes, n) == _depth_recursive(nodes)


def test_tree_depth_of_identical_triangles(oracle):
    # 64 identical triangles: one Morton code, midpoint splits, depth log2(64)
    v = np.tile(sc.triangle_soup(1, seed_salt=410), (64, 1))
    assert ref_gpu.tree_depth(oracle.lbvh(v)["ref_nodes"], 64) == 6


def test_config2_tree_fits_the_reference_stack(oracle):
    v = sc.triangle_soup(1000000)
    d = ref_gpu.tree_depth(oracle.lbvh(v)["ref_nodes"], 1000000)
    assert d <= ref_gpu.STACK_ENTRIES


@pytest.mark.parametrize("damage", ["child", "leaf_index", "count", "shared_child"])
def test_tree_depth_rejects_indices_out_of_range(oracle, damage):
    n = 100
    nodes = oracle.lbvh(sc.triangle_soup(n, seed_salt=420))["ref_nodes"].copy()
    w = nodes.reshape(-1, 8)
    inner = np.nonzero((w[:, 7] & 0xFF) == 0)[0]
    leaf = np.nonzero(w[:, 7] & 0xFF)[0]
    if damage == "child":
        w[inner[3], 6] = 2 * n + 5
    elif damage == "leaf_index":
        w[leaf[0], 6] = n
    elif damage == "count":
        nodes = nodes[:-8]
    else:
        # the root's right child pointed at a node inside its left subtree
        w[0, 6] = 2
    with pytest.raises(ValueError):
        ref_gpu.tree_depth(nodes, n)


def test_layout_file_when_built():
    if not os.path.exists(ref_gpu.LAYOUT):
        pytest.skip("reference kernels not built here")
    with open(ref_gpu.LAYOUT) as f:
        L = json.load(f)
    assert (L["ray_size"], L["hit_size"], L["hit_id"], L["node_size"]) == (32, 16, 4, 32)
    assert L["triangle_size"] % 8 == 0
    assert L["sv_bvh"] + 8 <= L["scene_view_size"]
    assert L["sv_triangles"] + 8 <= L["scene_view_size"]
    assert L["tri_index"] + 4 <= L["triangle_size"]
