"""Generates tests/golden/loader_ref.npz: what the reference's own scene loader
(Scene::Scene, src/renderer/scene.cpp:4-27, compiled from the reference sources
by oracle/ref/build_ref.sh into oracle/_ref/libref_loader.so) produces for

  - loader_shapes.xml (+ loader_tri.obj), this directory's fixture: the full
    arrays (triangles, normals, texture coordinates, mesh of each triangle,
    material records, camera, environment);
  - the reference's own scene/CBox/cbox.xml, cbox(mesh).xml and
    cbox(sphere).xml: the counts, SHA-256 digests of the triangle, normal,
    texture-coordinate and mesh arrays (the files themselves are the
    reference's and stay in its tree), and the small arrays in full.

Run where the reference tree is (GR_REFERENCE_ROOT) after
`python -c "import __graft_entry__ as g; g.build()"`:

    python tests/golden/make_golden_loader.py
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import refloader  # noqa: E402
import refsrc  # noqa: E402

FIXTURE = os.path.join(HERE, "loader_shapes.xml")
OUT = os.path.join(HERE, "loader_ref.npz")


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main():
    if not refloader.available():
        sys.exit("oracle/_ref/libref_loader.so is not built (needs the reference sources)")
    out = {}
    r = refloader.load(FIXTURE)
    for k, v in r.items():
        out["shapes_" + k] = v
    for name, path in sorted(refsrc.cbox_scenes().items()):
        key = name.replace(".xml", "").replace("(", "_").replace(")", "")
        r = refloader.load(path)
        out[key + "_counts"] = np.array([r["verts"].shape[0], r["materials"].shape[0]], np.int64)
        for k in ("verts", "normals", "uvs", "mesh"):
            out[key + "_sha_" + k] = np.array(digest(r[k]))
        for k in ("materials", "camera", "env"):
            out[key + "_" + k] = r[k]
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, sorted(out))


if __name__ == "__main__":
    main()
