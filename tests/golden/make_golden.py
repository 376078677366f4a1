"""Generates tests/golden/lbvh_ref.npz by running the reference's own host
LBVH_build (src/renderer/bvh.h:186-221, compiled from the reference sources by
oracle/ref/build_ref.sh into oracle/_ref/) on small seeded triangle soups.

Run from the repository root where the reference sources exist:
    bash oracle/ref/build_ref.sh && python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "gpu-renderer_gb300"))
import pyoracle  # noqa: E402
from gr import scenes  # noqa: E402


def cases():
    out = {}
    out["n1"] = scenes.triangle_soup(1, seed_salt=11)
    out["n2"] = scenes.triangle_soup(2, seed_salt=12)
    out["n7"] = scenes.triangle_soup(7, seed_salt=13)
    v = scenes.triangle_soup(1000, seed_salt=14)
    v[500:520] = v[500]          # a run of 20 identical triangles
    v[10:13] = v[900]            # scattered duplicates of one triangle
    out["soup1000_dups"] = v
    out["all_same"] = np.repeat(scenes.triangle_soup(1, seed_salt=15), 64, axis=0)
    f = scenes.triangle_soup(256, seed_salt=16).reshape(256, 3, 3)
    f[:, :, 2] = 0.5             # every centroid on one plane: a zero-extent axis
    out["flat"] = f.reshape(256, 9).copy()
    out["soup4096"] = scenes.triangle_soup(4096, seed_salt=17)
    return out


def main():
    if not pyoracle.ref_available():
        raise SystemExit("oracle/_ref/libref_lbvh.so missing: run oracle/ref/build_ref.sh first")
    data = {}
    for name, v in cases().items():
        nodes, codes = pyoracle.ref_lbvh(v)
        data[name + "/verts"] = v
        data[name + "/ref_nodes"] = nodes
        data[name + "/codes"] = codes
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lbvh_ref.npz")
    np.savez_compressed(path, **data)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
