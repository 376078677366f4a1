"""Where the reference's sources are, for the build recipes and the fixture
generators that compile or read them (test infrastructure; nothing in the
product uses it).

One environment variable, GR_REFERENCE_ROOT, names the reference tree; its
default is the location the build container mounts it at. On machines without
it (the GPU machine) every user of this module skips what needs the tree.
"""
import os

REFERENCE_ROOT = os.environ.get("GR_REFERENCE_ROOT", "/root/reference")


def root():
    """The reference tree, or None when its sources are absent."""
    return REFERENCE_ROOT if os.path.isfile(os.path.join(REFERENCE_ROOT, "src", "renderer", "bvh.h")) else None


def path(*parts):
    """A path inside the reference tree, or None when the tree is absent."""
    r = root()
    return os.path.join(r, *parts) if r else None


def cbox_scenes():
    """The reference's Cornell-box fixtures (scene/CBox/*.xml) by file name,
    {} when the tree is absent."""
    d = path("scene", "CBox")
    if not d or not os.path.isdir(d):
        return {}
    return {n: os.path.join(d, n) for n in ("cbox.xml", "cbox(mesh).xml", "cbox(sphere).xml")
            if os.path.exists(os.path.join(d, n))}
