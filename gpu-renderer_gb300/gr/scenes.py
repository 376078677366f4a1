"""Seeded synthetic inputs for the benchmark configurations.

Every generator uses numpy's PCG64 stream seeded with 0x5EED0000 + config
number, and stores geometry as float32 triangle soups (9 floats per triangle)
and rays as 8 floats (o.xyz, d.xyz, tmin, tmax), the reference's Ray layout.
"""
import numpy as np

SEED_BASE = 0x5EED0000


def rng(config, salt=0):
    return np.random.Generator(np.random.PCG64(SEED_BASE + config + (salt << 8)))


def _unit_vectors(r, shape):
    u = r.standard_normal(size=shape + (3,)).astype(np.float32)
    u /= np.linalg.norm(u, axis=-1, keepdims=True)
    return u


def triangle_soup(n, seed_salt=0, config=2):
    """Config 2 geometry: n triangles with centroids uniform in the unit cube,
    vertex offsets of lognormal length (mu=-6, sigma=0.5) in random
    directions."""
    r = rng(config, seed_salt)
    c = r.random((n, 3), dtype=np.float32)
    s = np.exp(r.normal(-6.0, 0.5, size=(n, 3))).astype(np.float32)
    u = _unit_vectors(r, (n, 3))
    v = c[:, None, :] + s[:, :, None] * u
    return np.ascontiguousarray(v.reshape(n, 9), dtype=np.float32)


def incoherent_rays(m, seed_salt=1, config=2):
    """Origins uniform in the unit cube, directions uniform on the sphere,
    tMin 0, tMax 1e34 (the camera-ray convention)."""
    r = rng(config, seed_salt)
    o = r.random((m, 3), dtype=np.float32)
    d = _unit_vectors(r, (m,))
    R = np.empty((m, 8), np.float32)
    R[:, 0:3] = o
    R[:, 3:6] = d
    R[:, 6] = 0.0
    R[:, 7] = 1e34
    return R


def shadow_rays(m, seed_salt=2, config=2):
    """Any-hit rays: d = p2 - o to a second uniform point, tMin 0, tMax 0.9999
    (the shadow-ray convention of the reference's NEE)."""
    r = rng(config, seed_salt)
    o = r.random((m, 3), dtype=np.float32)
    p2 = r.random((m, 3), dtype=np.float32)
    R = np.empty((m, 8), np.float32)
    R[:, 0:3] = o
    R[:, 3:6] = p2 - o
    R[:, 6] = 0.0
    R[:, 7] = np.float32(0.9999)
    return R


def coherent_rays(w=2048, h=2048, fov_deg=40.0, eye=(0.5, 0.5, -1.0), target=(0.5, 0.5, 0.5)):
    """Pixel-centre pinhole rays over a w x h grid."""
    eye = np.asarray(eye, np.float64)
    fwd = np.asarray(target, np.float64) - eye
    fwd /= np.linalg.norm(fwd)
    up = np.array([0.0, 1.0, 0.0])
    right = np.cross(fwd, up)
    right /= np.linalg.norm(right)
    upv = np.cross(right, fwd)
    tan = np.tan(np.radians(fov_deg) * 0.5)
    aspect = w / h
    xs = ((np.arange(w) + 0.5) / w * 2.0 - 1.0) * tan * aspect
    ys = (1.0 - (np.arange(h) + 0.5) / h * 2.0) * tan
    X, Y = np.meshgrid(xs, ys)
    d = fwd[None, None, :] + X[..., None] * right[None, None, :] + Y[..., None] * upv[None, None, :]
    d /= np.linalg.norm(d, axis=-1, keepdims=True)
    R = np.empty((h * w, 8), np.float32)
    R[:, 0:3] = eye.astype(np.float32)
    R[:, 3:6] = d.reshape(-1, 3).astype(np.float32)
    R[:, 6] = 0.0
    R[:, 7] = 1e34
    return R
