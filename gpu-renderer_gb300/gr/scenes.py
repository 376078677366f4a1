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


def surface_rays(soup, m, seed_salt=3, config=1, tmin=1e-4):
    """Secondary-ray-like queries: origins uniform on random triangles of the
    soup, directions uniform on the sphere with half of them squeezed towards
    an axis plane (one component scaled by 1e-3, then renormalised), tmin 1e-4.
    These start on surfaces and graze axis-aligned walls, where a plane
    distance with an absolute rounding error would cull a hit box."""
    r = rng(config, seed_salt)
    v = np.asarray(soup, np.float32).reshape(-1, 3, 3)
    t = r.integers(0, v.shape[0], m)
    a, b = r.random(m), r.random(m)
    sa = np.sqrt(a)
    w = np.stack([1 - sa, sa * (1 - b), sa * b], axis=1)
    p = np.einsum("mk,mkc->mc", w, v[t].astype(np.float64)).astype(np.float32)
    d = r.standard_normal((m, 3))
    g = r.random(m) < 0.5
    ax = r.integers(0, 3, m)
    d[g, ax[g]] *= 1e-3
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    R = np.empty((m, 8), np.float32)
    R[:, 0:3] = p
    R[:, 3:6] = d
    R[:, 6] = np.float32(tmin)
    R[:, 7] = np.float32(1e38)
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


# ---- scene descriptions for the render configurations -----------------------------

class MeshDesc:
    def __init__(self, positions, indices, material, normals=None, texcoords=None):
        self.positions = np.ascontiguousarray(positions, np.float32).reshape(-1, 3)
        self.indices = np.ascontiguousarray(indices, np.uint32).reshape(-1, 3)
        self.normals = None if normals is None else np.ascontiguousarray(normals, np.float32).reshape(-1, 3)
        self.texcoords = None if texcoords is None else np.ascontiguousarray(texcoords, np.float32).reshape(-1, 2)
        self.material = int(material)


class SceneDesc:
    """Meshes + materials (dicts for gr.material_record) + camera +
    environment: None, a constant radiance (3 floats), or a dict
    {"map": (H, W, 3) float32 rows bottom first, "to_world": 4x4}."""

    def __init__(self, meshes, materials, camera, env=None):
        self.meshes = meshes
        self.materials = materials
        self.camera = camera
        self.env = env

    @property
    def num_triangles(self):
        return sum(m.indices.shape[0] for m in self.meshes)

    def flatten(self):
        """Triangle soup, per-corner normals, material words, in the order the
        library flattens them (mesh order, then triangle order)."""
        n = self.num_triangles
        soup = np.zeros((n, 9), np.float32)
        nrm = np.zeros((n, 12), np.float32)
        tmat = np.zeros(n, np.uint32)
        t = 0
        for m in self.meshes:
            k = m.indices.shape[0]
            soup[t:t + k] = m.positions[m.indices].reshape(k, 9)
            if m.normals is not None:
                nn = m.normals[m.indices]  # (k, 3, 3)
                nrm[t:t + k].reshape(k, 3, 4)[:, :, :3] = nn
                tmat[t:t + k] = m.material | 0x80000000
            else:
                tmat[t:t + k] = m.material
            t += k
        any_n = any(m.normals is not None for m in self.meshes)
        return soup, (nrm if any_n else None), tmat

    def flatten_uv(self):
        """Per-triangle corner texcoords (n, 6) and the texcoord flag bits
        (0x40000000 per triangle that has them), or (None, zeros)."""
        n = self.num_triangles
        uv = np.zeros((n, 6), np.float32)
        bits = np.zeros(n, np.uint32)
        t = 0
        for m in self.meshes:
            k = m.indices.shape[0]
            if m.texcoords is not None:
                uv[t:t + k] = m.texcoords[m.indices].reshape(k, 6)
                bits[t:t + k] = 0x40000000
            t += k
        return (uv if bits.any() else None), bits


def look_at(origin, target, up):
    """Camera-to-world matrix of the reference's LookAt (transform.cpp:220-249):
    columns left, up, forward, origin; row-major 4x4 float32."""
    o = np.asarray(origin, np.float32)
    f = np.asarray(target, np.float32) - o
    f = f / np.sqrt(np.float32(np.dot(f, f)))
    left = np.cross(np.asarray(up, np.float32), f).astype(np.float32)
    left = left / np.sqrt(np.float32(np.dot(left, left)))
    u = np.cross(f, left).astype(np.float32)
    M = np.eye(4, dtype=np.float32)
    M[:3, 0] = left
    M[:3, 1] = u
    M[:3, 2] = f
    M[:3, 3] = o
    return M


def quad(p0, p1, p2, p3):
    """Two triangles (p0, p1, p2), (p0, p2, p3); geometric normal follows the
    reference's cross(p0 - p2, p1 - p2) of the first triangle."""
    P = np.array([p0, p1, p2, p3], np.float32)
    return P, np.array([[0, 1, 2], [0, 2, 3]], np.uint32)


def box_mesh(center, size, yaw):
    """12-triangle axis box, rotated by `yaw` about +y."""
    sx, sy, sz = size
    c = np.array(center, np.float32)
    corners = np.array([[x, y, z] for x in (-0.5, 0.5) for y in (0.0, 1.0) for z in (-0.5, 0.5)], np.float32)
    corners *= np.array([sx, sy, sz], np.float32)
    cy, syw = np.cos(yaw), np.sin(yaw)
    R = np.array([[cy, 0, syw], [0, 1, 0], [-syw, 0, cy]], np.float32)
    P = (corners @ R.T + c).astype(np.float32)
    # corner index = 4*ix + 2*iy + iz
    faces = [(0, 1, 3, 2), (4, 6, 7, 5), (0, 4, 5, 1), (2, 3, 7, 6), (0, 2, 6, 4), (1, 5, 7, 3)]
    idx = []
    for a, b, cc, d in faces:
        idx += [[a, b, cc], [a, cc, d]]
    return P, np.array(idx, np.uint32)


def cornell_box(width=256, height=256, seed_salt=0):
    """Config 1: procedural Cornell box. Five walls as 10 triangles (floor,
    ceiling, back grey 0.75; left red 0.63/0.065/0.05; right green
    0.14/0.45/0.09), a 2-triangle quad light of radiance 15 below the ceiling,
    and two 12-triangle boxes rotated by a seeded yaw. Lambert everywhere;
    pinhole camera with a 40 degree field of view."""
    r = rng(1, seed_salt)
    grey = {"type": 0, "color": (0.75, 0.75, 0.75)}
    red = {"type": 0, "color": (0.63, 0.065, 0.05)}
    green = {"type": 0, "color": (0.14, 0.45, 0.09)}
    light = {"type": 0, "color": (0.75, 0.75, 0.75), "emission": (15.0, 15.0, 15.0)}
    mats = [grey, red, green, light]
    meshes = []
    walls = [
        (quad((-1, 0, -1), (1, 0, -1), (1, 0, 1), (-1, 0, 1)), 0),     # floor
        (quad((-1, 2, -1), (-1, 2, 1), (1, 2, 1), (1, 2, -1)), 0),     # ceiling
        (quad((-1, 0, -1), (-1, 2, -1), (1, 2, -1), (1, 0, -1)), 0),   # back
        (quad((-1, 0, -1), (-1, 0, 1), (-1, 2, 1), (-1, 2, -1)), 1),   # left
        (quad((1, 0, -1), (1, 2, -1), (1, 2, 1), (1, 0, 1)), 2),       # right
    ]
    for (P, I), mi in walls:
        meshes.append(MeshDesc(P, I, mi))
    # light quad facing down: cross(p0 - p2, p1 - p2) points to -y
    LP, LI = quad((-0.25, 1.98, -0.25), (0.25, 1.98, -0.25), (0.25, 1.98, 0.25), (-0.25, 1.98, 0.25))
    meshes.append(MeshDesc(LP, LI, 3))
    yaw = r.random(2) * 2.0 * np.pi
    for center, size, yw in (((-0.35, 0.0, -0.35), (0.6, 1.2, 0.6), yaw[0]),
                             ((0.35, 0.0, 0.3), (0.6, 0.6, 0.6), yaw[1])):
        P, I = box_mesh(center, size, yw)
        meshes.append(MeshDesc(P, I, 0))
    cam = {"to_world": look_at((0.0, 1.0, 3.8), (0.0, 1.0, 0.0), (0.0, 1.0, 0.0)), "fov": 40.0,
           "width": width, "height": height}
    return SceneDesc(meshes, mats, cam, env=None)


_ICO_CACHE = {}


def icosphere(level):
    """Unit icosphere: 20 * 4^level triangles with shared vertices (cached)."""
    if level in _ICO_CACHE:
        V, F = _ICO_CACHE[level]
        return V.copy(), F.copy()
    V, F = _icosphere(level)
    _ICO_CACHE[level] = (V, F)
    return V.copy(), F.copy()


def _icosphere(level):
    t = (1.0 + 5.0 ** 0.5) / 2.0
    V = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], np.float64)
    V /= np.linalg.norm(V, axis=1, keepdims=True)
    F = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2],
                  [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5],
                  [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], np.int64)
    for _ in range(level):
        e = np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]])
        e.sort(axis=1)
        uniq, inv = np.unique(e, axis=0, return_inverse=True)
        mid = V[uniq[:, 0]] + V[uniq[:, 1]]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        base = V.shape[0]
        V = np.concatenate([V, mid])
        nf = F.shape[0]
        inv = inv.reshape(-1)
        m01, m12, m20 = inv[:nf] + base, inv[nf:2 * nf] + base, inv[2 * nf:] + base
        F = np.concatenate([np.stack([F[:, 0], m01, m20], 1), np.stack([F[:, 1], m12, m01], 1),
                            np.stack([F[:, 2], m20, m12], 1), np.stack([m01, m12, m20], 1)])
    return V, F


def value_noise3(p, seed, octaves=3):
    """Seeded 3-octave value noise on points p (N, 3): hashed lattice values in
    [-1, 1], smoothstep-trilinear interpolation, frequency doubling and
    amplitude halving per octave; result roughly in [-1, 1]."""
    out = np.zeros(p.shape[0], np.float64)
    amp, freq, norm = 1.0, 2.0, 0.0
    for o in range(octaves):
        q = p * freq
        i0 = np.floor(q).astype(np.int64)
        f = q - i0
        f = f * f * (3.0 - 2.0 * f)
        acc = np.zeros(p.shape[0])
        for dx in (0, 1):
            for dy in (0, 1):
                for dz in (0, 1):
                    h = (i0[:, 0] + dx) * 73856093 ^ (i0[:, 1] + dy) * 19349663 ^ (i0[:, 2] + dz) * 83492791
                    h = (h ^ (seed * 2654435761 + o * 97531)) & 0xFFFFFFFF
                    h = (h * 2246822519) & 0xFFFFFFFF
                    h ^= h >> 13
                    h = (h * 3266489917) & 0xFFFFFFFF
                    h ^= h >> 16
                    v = (h / 4294967295.0) * 2.0 - 1.0
                    w = (f[:, 0] if dx else 1 - f[:, 0]) * (f[:, 1] if dy else 1 - f[:, 1]) * \
                        (f[:, 2] if dz else 1 - f[:, 2])
                    acc += w * v
        out += amp * acc
        norm += amp
        amp *= 0.5
        freq *= 2.0
    return out / norm


def displaced_sphere(level, radius, center, amplitude, seed):
    """Icosphere radially displaced by value noise; vertex normals are
    normalised sums of adjacent face normals."""
    V, F = icosphere(level)
    disp = 1.0 + amplitude * value_noise3(V, seed)
    P = V * disp[:, None] * radius + np.asarray(center, np.float64)
    fn = np.cross(P[F[:, 1]] - P[F[:, 0]], P[F[:, 2]] - P[F[:, 0]])
    N = np.zeros_like(P)
    for c in range(3):
        for k in range(3):
            N[:, c] += np.bincount(F[:, k], weights=fn[:, c], minlength=P.shape[0])
    N /= np.linalg.norm(N, axis=1, keepdims=True)
    return P.astype(np.float32), F.astype(np.uint32), N.astype(np.float32)


def glossy_scene(width=1024, height=768, level=8, glass_level=5, seed_salt=0):
    """Config 3: four noise-displaced icospheres (level 8 = 1,310,720 triangles
    each, amplitude 0.05) with GGX conductors of roughness 0.01 / 0.1 / 0.25 /
    0.5 (Cu-like eta/k, the reference's defaults), one smooth dielectric sphere
    (IOR 1.5, icosphere level 5 = 20,480 triangles), a 2-triangle ground plane,
    a constant environment and one quad light."""
    mats = [
        {"type": 0, "color": (0.5, 0.5, 0.5)},                                   # ground
        {"type": 0, "color": (0.5, 0.5, 0.5), "emission": (20.0, 20.0, 20.0)},   # light
        {"type": 1, "color": (1.0, 1.0, 1.0), "ior": 1.5},                       # glass
    ]
    alphas = (0.01, 0.1, 0.25, 0.5)
    for a in alphas:
        mats.append({"type": 2, "color": (1.0, 1.0, 1.0), "alpha": a})
    meshes = []
    GP, GI = quad((-10, 0, -10), (-10, 0, 10), (10, 0, 10), (10, 0, -10))
    meshes.append(MeshDesc(GP, GI, 0))
    LP, LI = quad((-0.5, 3.0, -0.5), (0.5, 3.0, -0.5), (0.5, 3.0, 0.5), (-0.5, 3.0, 0.5))
    meshes.append(MeshDesc(LP, LI, 1))
    for i, x in enumerate((-1.65, -0.55, 0.55, 1.65)):
        P, F, N = displaced_sphere(level, 0.5, (x, 0.55, 0.0), 0.05, seed=SEED_BASE + 3 + i + (seed_salt << 4))
        meshes.append(MeshDesc(P, F, 3 + i, normals=N))
    P, F, N = displaced_sphere(glass_level, 0.4, (0.0, 0.4, 1.1), 0.0, seed=1)
    meshes.append(MeshDesc(P, F, 2, normals=N))
    cam = {"to_world": look_at((0.0, 1.3, 4.6), (0.0, 0.5, 0.0), (0.0, 1.0, 0.0)), "fov": 40.0,
           "width": width, "height": height}
    return SceneDesc(meshes, mats, cam, env=(0.3, 0.35, 0.45))


_DISPLACED_CACHE = {}


def _unit_displaced(level, variant):
    """Unit icosphere displaced by seeded 3-octave value noise (amplitude 0.05),
    cached by (level, variant)."""
    key = (level, variant)
    if key not in _DISPLACED_CACHE:
        _DISPLACED_CACHE[key] = displaced_sphere(level, 1.0, (0.0, 0.0, 0.0), 0.05, seed=SEED_BASE + 977 * variant + level)
    return _DISPLACED_CACHE[key]


RESOLUTIONS = (128, 256, 512, 1024)
SPPS = (4, 16, 64)


def batch_job(index, config=4, min_tris=10_000, max_tris=2_000_000):
    """Config 4 job `index`: a seeded scene with a log-uniform triangle count in
    [10k, 2M], built from noise-displaced icospheres (levels 5-8) and boxes
    with Lambert, GGX-conductor or dielectric materials, on a ground plane
    with one quad light and a constant environment. Returns (SceneDesc, spp)
    with a resolution drawn from {128, 256, 512, 1024}^2 and spp from {4, 16, 64}."""
    r = rng(config, index + 1)
    target = int(np.exp(r.uniform(np.log(min_tris), np.log(max_tris))))
    res = int(r.choice(RESOLUTIONS))
    spp = int(r.choice(SPPS))
    mats = [{"type": 0, "color": (0.6, 0.6, 0.6)},
            {"type": 0, "color": (0.5, 0.5, 0.5), "emission": (12.0, 12.0, 12.0)}]
    meshes = []
    GP, GI = quad((-6, 0, -6), (-6, 0, 6), (6, 0, 6), (6, 0, -6))
    meshes.append(MeshDesc(GP, GI, 0))
    LP, LI = quad((-0.6, 4.0, -0.6), (0.6, 4.0, -0.6), (0.6, 4.0, 0.6), (-0.6, 4.0, 0.6))
    meshes.append(MeshDesc(LP, LI, 1))

    def add_material():
        kind = int(r.integers(0, 3))
        if kind == 0:
            mats.append({"type": 0, "color": tuple(float(x) for x in r.uniform(0.2, 0.9, 3))})
        elif kind == 1:
            mats.append({"type": 2, "color": (1.0, 1.0, 1.0), "alpha": float(r.choice((0.01, 0.1, 0.25, 0.5)))})
        else:
            mats.append({"type": 1, "color": (1.0, 1.0, 1.0), "ior": 1.5})
        return len(mats) - 1

    remaining = target - 4
    while remaining >= 20 * 4 ** 5:
        level = 5
        while level < 8 and 20 * 4 ** (level + 1) <= remaining:
            level += 1
        if level > 5 and r.random() < 0.3:
            level -= 1
        P, F, N = _unit_displaced(level, int(r.integers(0, 4)))
        radius = float(r.uniform(0.3, 0.8))
        center = (float(r.uniform(-2.5, 2.5)), radius * 1.05, float(r.uniform(-2.5, 1.5)))
        meshes.append(MeshDesc(P * radius + np.asarray(center, np.float32), F, add_material(), normals=N))
        remaining -= F.shape[0]
    nbox = max(1, remaining // 12)
    boxes_p, boxes_i = [], []
    m_box = add_material()
    for b in range(nbox):
        s = r.uniform(0.05, 0.4, 3)
        c = (float(r.uniform(-3, 3)), 0.0, float(r.uniform(-3, 2)))
        P, I = box_mesh(c, s, float(r.uniform(0, 2 * np.pi)))
        boxes_i.append(I + 8 * b)
        boxes_p.append(P)
    meshes.append(MeshDesc(np.concatenate(boxes_p), np.concatenate(boxes_i), m_box))
    cam = {"to_world": look_at((0.0, 2.2, 6.5), (0.0, 0.6, 0.0), (0.0, 1.0, 0.0)), "fov": 45.0,
           "width": res, "height": res}
    return SceneDesc(meshes, mats, cam, env=(0.25, 0.3, 0.35)), spp


def checker_map(c0, c1):
    """The reference's checkerboard texture: the 2 x 2 map (c0, c1; c1, c0)."""
    return np.array([[c0, c1], [c1, c0]], np.float32)


def textured_scene(width=64, height=48, seed_salt=0):
    """Textures and an environment map: a checkerboard ground quad with
    texcoords (uv scale 6, offset 0.25), a Lambert icosphere with a seeded
    16 x 8 bitmap looked up at its barycentrics (no texcoords), a GGX conductor
    icosphere with a checkerboard specular colour, a quad light, and a seeded
    64 x 32 latitude-longitude environment map rotated about the vertical."""
    r = rng(6, seed_salt)
    mats = [
        {"type": 0, "color": (0.5, 0.5, 0.5), "color_map": checker_map((0.8, 0.8, 0.8), (0.1, 0.2, 0.5)),
         "uv_scale": (6.0, 6.0), "uv_offset": (0.25, 0.25)},
        {"type": 0, "color": (0.5, 0.5, 0.5), "color_map": r.uniform(0.05, 0.95, (8, 16, 3)).astype(np.float32)},
        {"type": 2, "color": (1.0, 1.0, 1.0), "alpha": 0.2,
         "color_map": checker_map((1.0, 0.8, 0.3), (0.4, 0.9, 1.0)), "uv_scale": (3.0, 3.0)},
        {"type": 0, "color": (0.5, 0.5, 0.5), "emission": (20.0, 20.0, 20.0)},
    ]
    GP, GI = quad((-4, 0, -4), (-4, 0, 4), (4, 0, 4), (4, 0, -4))
    GT = np.array([[0, 0], [0, 1], [1, 1], [1, 0]], np.float32)
    V, F = icosphere(2)
    LP, LI = quad((-0.5, 3.0, -0.5), (0.5, 3.0, -0.5), (0.5, 3.0, 0.5), (-0.5, 3.0, 0.5))
    meshes = [MeshDesc(GP, GI, 0, texcoords=GT),
              MeshDesc(V * 0.7 + np.array([-0.8, 0.7, 0.0]), F, 1),
              MeshDesc(V * 0.6 + np.array([0.9, 0.6, 0.3]), F, 2),
              MeshDesc(LP, LI, 3)]
    ang = 0.7
    rot = np.array([[np.cos(ang), 0, np.sin(ang), 0], [0, 1, 0, 0], [-np.sin(ang), 0, np.cos(ang), 0], [0, 0, 0, 1]],
                   np.float32)
    yy, xx = np.mgrid[0:32, 0:64]
    env = np.stack([0.3 + 0.6 * xx / 63.0, 0.2 + 0.7 * yy / 31.0, 0.8 - 0.5 * yy / 31.0], axis=-1).astype(np.float32)
    env += r.uniform(0.0, 0.1, env.shape).astype(np.float32)
    cam = {"to_world": look_at((0.0, 2.0, 6.0), (0.0, 0.6, 0.0), (0.0, 1.0, 0.0)), "fov": 45.0,
           "width": width, "height": height}
    return SceneDesc(meshes, mats, cam, {"map": env, "to_world": rot})


def plastic_scene(width=64, height=48, seed_salt=0):
    """Rough plastic (Lambert + GGX lobes with dielectric Fresnel) at three
    roughnesses on a grey ground under a quad light and a constant
    environment."""
    mats = [{"type": 0, "color": (0.6, 0.6, 0.6)},
            {"type": 0, "color": (0.5, 0.5, 0.5), "emission": (15.0, 15.0, 15.0)}]
    meshes = []
    GP, GI = quad((-4, 0, -4), (-4, 0, 4), (4, 0, 4), (4, 0, -4))
    meshes.append(MeshDesc(GP, GI, 0))
    LP, LI = quad((-0.5, 3.0, -0.5), (0.5, 3.0, -0.5), (0.5, 3.0, 0.5), (-0.5, 3.0, 0.5))
    meshes.append(MeshDesc(LP, LI, 1))
    V, F = icosphere(3)
    for k, (alpha, col) in enumerate(((0.05, (0.8, 0.2, 0.1)), (0.2, (0.1, 0.5, 0.8)), (0.5, (0.3, 0.7, 0.2)))):
        mats.append({"type": 3, "color": col, "specular": (1.0, 1.0, 1.0), "alpha": alpha,
                     "eta_i": (1.5, 1.5, 1.5), "eta_t": (1.0, 1.0, 1.0)})
        meshes.append(MeshDesc(V * 0.55 + np.array([-1.3 + 1.3 * k, 0.55, 0.0]), F, len(mats) - 1))
    cam = {"to_world": look_at((0.0, 1.8, 5.0), (0.0, 0.5, 0.0), (0.0, 1.0, 0.0)), "fov": 45.0,
           "width": width, "height": height}
    return SceneDesc(meshes, mats, cam, (0.2, 0.2, 0.25))
