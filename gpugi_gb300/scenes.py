"""Seeded synthetic scenes and ray sets.

gpugi loads its geometry from `.bim` files that are not part of the
reference snapshot, so every workload here is generated from a seed. All
randomness comes from a counter-based splitmix64 hash (vectorised in numpy
uint64 arithmetic), so the same seed gives the same arrays on every machine.

A scene is a dict of numpy arrays:
  positions  float32 [V, 3]
  normals    float32 [V, 3]   (unit shading normals)
  texcoords  float32 [V, 2]
  triangles  uint32  [T, 4]   {v0, v1, v2, material}
  materials  float32 [M, 24]  material records (see `material_record`)
  plus optional light descriptions used by the renderers.
"""
from __future__ import annotations

import math

import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _splitmix64(x: np.ndarray) -> np.ndarray:
    """splitmix64 finaliser on a uint64 array (Steele, Lea, Flood 2014)."""
    with np.errstate(over="ignore"):
        z = (x + np.uint64(0x9E3779B97F4A7C15)) & _M64
        z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & _M64
        z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & _M64
        return z ^ (z >> np.uint64(31))


class Stream:
    """A counter-based random stream: stream(seed, tag) draws are reproducible."""

    def __init__(self, seed: int, tag: int = 0):
        self._key = int(_splitmix64(np.array([(seed * 0x100000001B3 + tag) & 0xFFFFFFFFFFFFFFFF],
                                             dtype=np.uint64))[0])
        self._ctr = 0

    def u64(self, n: int) -> np.ndarray:
        idx = np.arange(self._ctr, self._ctr + n, dtype=np.uint64)
        self._ctr += n
        with np.errstate(over="ignore"):
            return _splitmix64((idx * np.uint64(0xD1342543DE82EF95)) ^ np.uint64(self._key))

    def uniform(self, n: int, lo: float = 0.0, hi: float = 1.0) -> np.ndarray:
        """float64 uniform in [lo, hi) with 53 random bits."""
        u = (self.u64(n) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
        return lo + (hi - lo) * u

    def unit_vectors(self, n: int) -> np.ndarray:
        """Uniform directions on the sphere by rejection from the cube (no transcendental calls)."""
        out = np.empty((0, 3), dtype=np.float64)
        while out.shape[0] < n:
            m = 2 * (n - out.shape[0]) + 64
            c = self.uniform(3 * m, -1.0, 1.0).reshape(m, 3)
            r2 = np.einsum("ij,ij->i", c, c)
            keep = (r2 <= 1.0) & (r2 > 1e-6)
            out = np.concatenate([out, c[keep] / np.sqrt(r2[keep])[:, None]])
        return out[:n]

    def quaternions(self, n: int) -> np.ndarray:
        out = np.empty((0, 4), dtype=np.float64)
        while out.shape[0] < n:
            m = 3 * (n - out.shape[0]) + 64
            c = self.uniform(4 * m, -1.0, 1.0).reshape(m, 4)
            r2 = np.einsum("ij,ij->i", c, c)
            keep = (r2 <= 1.0) & (r2 > 1e-6)
            out = np.concatenate([out, c[keep] / np.sqrt(r2[keep])[:, None]])
        return out[:n]


def quat_to_matrix(q: np.ndarray) -> np.ndarray:
    w, x, y, z = q[..., 0], q[..., 1], q[..., 2], q[..., 3]
    return np.stack([
        np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)], -1),
        np.stack([2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)], -1),
        np.stack([2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], -1),
    ], -2)


# --------------------------------------------------------------------------
# Materials
# --------------------------------------------------------------------------
MATERIAL_FLOATS = 24  # 6 x float4, see include/gpugi_cuda.h (gpugi_material)


def material_record(albedo=(0.5, 0.5, 0.5), emissivity=(0.0, 0.0, 0.0), specular=(0.0, 0.0, 0.0),
                    roughness: float = 1.0, opacity=(1.0, 1.0, 1.0), refraction_index: float = 1.5,
                    reflectiveness=(1.0, 1.0, 1.0)) -> np.ndarray:
    """Constant-valued material in the device layout.

    Mirrors the JSON-to-GPU mapping of Scene::LoadMaterial
    (gpugi/scene/scene.cpp:155-179): fresnel0 = specularColor,
    fresnel1 = 1 - fresnel0, Phong exponent = 1 / (roughness^2 + 1e-20),
    reflectiveness.w = exponent. Textures are replaced by their constant value.
    """
    exponent = np.float32(1.0) / (np.float32(roughness) * np.float32(roughness) + np.float32(1e-20))
    f0 = np.asarray(specular, dtype=np.float32)
    rec = np.zeros(MATERIAL_FLOATS, dtype=np.float32)
    rec[0:3] = albedo
    rec[3] = refraction_index
    rec[4:7] = opacity
    rec[8:11] = reflectiveness
    rec[11] = exponent
    rec[12:15] = emissivity
    rec[16:19] = f0
    rec[20:23] = np.float32(1.0) - f0
    return rec


def lambert(albedo, emissivity=(0.0, 0.0, 0.0)) -> np.ndarray:
    """A purely diffuse material: no Phong reflection (specularColor = 0)."""
    return material_record(albedo=albedo, emissivity=emissivity, specular=(0.0, 0.0, 0.0))


# --------------------------------------------------------------------------
# Meshes
# --------------------------------------------------------------------------
def icosphere(level: int):
    """Unit icosphere. Triangle order: level by level, every triangle
    (a, b, c) is replaced by (a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
             (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
             (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5),
             (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    v = np.array(verts, dtype=np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array(faces, dtype=np.int64)
    for _ in range(level):
        edges = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
        key = np.minimum(edges[:, 0], edges[:, 1]) * (1 << 32) + np.maximum(edges[:, 0], edges[:, 1])
        uniq, first, inv = np.unique(key, return_index=True, return_inverse=True)
        # midpoints get indices in order of first appearance
        order = np.argsort(first, kind="stable")
        rank = np.empty_like(order)
        rank[order] = np.arange(order.size)
        mid_idx = v.shape[0] + rank[inv]
        e = edges[first[order]]
        mids = v[e[:, 0]] + v[e[:, 1]]
        mids /= np.linalg.norm(mids, axis=1, keepdims=True)
        v = np.concatenate([v, mids])
        nf = f.shape[0]
        ab, bc, ca = mid_idx[:nf], mid_idx[nf:2 * nf], mid_idx[2 * nf:]
        a, b, c = f[:, 0], f[:, 1], f[:, 2]
        f = np.stack([np.stack([a, ab, ca], 1), np.stack([b, bc, ab], 1), np.stack([c, ca, bc], 1),
                      np.stack([ab, bc, ca], 1)], 1).reshape(-1, 3)
    return v, f


def box_mesh():
    """Unit cube [-0.5, 0.5]^3 as 12 outward-facing triangles."""
    v = np.array([[x, y, z] for x in (-0.5, 0.5) for y in (-0.5, 0.5) for z in (-0.5, 0.5)], dtype=np.float64)
    f = np.array([[0, 1, 3], [0, 3, 2], [4, 6, 7], [4, 7, 5], [0, 4, 5], [0, 5, 1],
                  [2, 3, 7], [2, 7, 6], [0, 2, 6], [0, 6, 4], [1, 5, 7], [1, 7, 3]], dtype=np.int64)
    return v, f


def torus_mesh(nu: int = 24, nv: int = 12, R: float = 0.35, r: float = 0.15):
    u = np.arange(nu) * (2 * math.pi / nu)
    w = np.arange(nv) * (2 * math.pi / nv)
    uu, ww = np.meshgrid(u, w, indexing="ij")
    v = np.stack([(R + r * np.cos(ww)) * np.cos(uu), (R + r * np.cos(ww)) * np.sin(uu), r * np.sin(ww)], -1)
    v = v.reshape(-1, 3)
    i, j = np.meshgrid(np.arange(nu), np.arange(nv), indexing="ij")
    a = i * nv + j
    b = ((i + 1) % nu) * nv + j
    c = ((i + 1) % nu) * nv + (j + 1) % nv
    d = i * nv + (j + 1) % nv
    f = np.concatenate([np.stack([a, b, c], -1).reshape(-1, 3), np.stack([a, c, d], -1).reshape(-1, 3)])
    return v, f


def vertex_normals(v: np.ndarray, f: np.ndarray) -> np.ndarray:
    fn = np.cross(v[f[:, 1]] - v[f[:, 0]], v[f[:, 2]] - v[f[:, 0]])
    n = np.zeros_like(v)
    for k in range(3):
        np.add.at(n, f[:, k], fn)
    ln = np.linalg.norm(n, axis=1, keepdims=True)
    ln[ln == 0] = 1.0
    return n / ln


def _pack(v, f, mats, material_ids=None, normals=None, texcoords=None, **extra):
    tris = np.zeros((f.shape[0], 4), dtype=np.uint32)
    tris[:, :3] = f
    if material_ids is not None:
        tris[:, 3] = material_ids
    if normals is None:
        normals = vertex_normals(v, f)
    if texcoords is None:
        texcoords = np.zeros((v.shape[0], 2))
    scene = dict(positions=np.ascontiguousarray(v, dtype=np.float32),
                 normals=np.ascontiguousarray(normals, dtype=np.float32),
                 texcoords=np.ascontiguousarray(texcoords, dtype=np.float32),
                 triangles=np.ascontiguousarray(tris),
                 materials=np.ascontiguousarray(np.asarray(mats, dtype=np.float32).reshape(-1, MATERIAL_FLOATS)))
    scene.update(extra)
    return scene


# --------------------------------------------------------------------------
# Workload 1: closest-hit queries against a displaced icosphere
# --------------------------------------------------------------------------
def displaced_icosphere(num_triangles: int = 65536, seed: int = 1, amplitude: float = 0.05):
    """Icosphere subdivided until it has >= num_triangles triangles, truncated
    to the first num_triangles in generation order, every vertex moved
    radially by uniform[-amplitude, amplitude], then scaled into the unit
    cube [0, 1]^3 (largest extent 1, centred in the cube).
    65,536 triangles = level 6 (81,920) truncated."""
    level = 0
    while 20 * 4 ** level < num_triangles:
        level += 1
    v, f = icosphere(level)
    f = f[:num_triangles]
    used, remap = np.unique(f, return_inverse=True)
    v = v[used]
    f = remap.reshape(-1, 3)
    rs = Stream(seed, 1)
    radius = 1.0 + rs.uniform(v.shape[0], -amplitude, amplitude)
    n = v.copy()
    v = v * radius[:, None]
    lo, hi = v.min(0), v.max(0)
    v = (v - (lo + hi) * 0.5) / (hi - lo).max() + 0.5
    return _pack(v, f, [lambert((0.5, 0.5, 0.5))], normals=n)


def closed_icosphere(level: int = 4, seed: int = 1, amplitude: float = 0.05):
    """A closed mesh: a level-`level` icosphere whose shared vertices are moved
    radially by uniform[-amplitude, amplitude], scaled into the unit cube and
    centred at (0.5, 0.5, 0.5) (star-shaped around the centre, so every ray
    from the centre must hit it)."""
    v, f = icosphere(level)
    rs = Stream(seed, 3)
    n = v.copy()
    v = v * (1.0 + rs.uniform(v.shape[0], -amplitude, amplitude))[:, None]
    lo, hi = v.min(0), v.max(0)
    v = (v - (lo + hi) * 0.5) / (hi - lo).max() + 0.5
    return _pack(v, f, [lambert((0.5, 0.5, 0.5))], normals=n)


def crack_rays(scene: dict, origin=(0.5, 0.5, 0.5)) -> dict:
    """Rays from `origin` through every vertex and every edge midpoint of a
    mesh: the rays a test that is not watertight can let slip between the
    triangles sharing that vertex or edge."""
    v = np.asarray(scene["positions"], np.float64)
    f = np.asarray(scene["triangles"])[:, :3].astype(np.int64)
    e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
    e = np.unique(np.sort(e, axis=1), axis=0)
    targets = np.concatenate([v, 0.5 * (v[e[:, 0]] + v[e[:, 1]])])
    d = targets - np.asarray(origin, np.float64)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    n = d.shape[0]
    o = np.asarray(origin, np.float32)
    return {"ox": np.full(n, o[0], np.float32), "oy": np.full(n, o[1], np.float32), "oz": np.full(n, o[2], np.float32),
            "dx": d[:, 0].astype(np.float32), "dy": d[:, 1].astype(np.float32), "dz": d[:, 2].astype(np.float32),
            "tmax": np.full(n, np.inf, np.float32)}


def aimed_rays(n: int, positions: np.ndarray, seed: int = 1, spread: float = 1.5, tmax: float = math.inf):
    """Rays from a box `spread` times the object's bounding box, each aimed at
    a uniform point of the object's bounding box (most of them hit)."""
    rs = Stream(seed, 3)
    lo, hi = positions.min(0).astype(np.float64), positions.max(0).astype(np.float64)
    c, h = (lo + hi) / 2, (hi - lo) / 2
    o = c + h * spread * rs.uniform(3 * n, -1.0, 1.0).reshape(n, 3)
    tgt = lo + (hi - lo) * rs.uniform(3 * n).reshape(n, 3)
    d = tgt - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    o = o.astype(np.float32)
    d = d.astype(np.float32)
    return dict(ox=np.ascontiguousarray(o[:, 0]), oy=np.ascontiguousarray(o[:, 1]),
                oz=np.ascontiguousarray(o[:, 2]), dx=np.ascontiguousarray(d[:, 0]),
                dy=np.ascontiguousarray(d[:, 1]), dz=np.ascontiguousarray(d[:, 2]),
                tmax=np.full(n, tmax, dtype=np.float32))


def random_rays(n: int, seed: int = 1, origin_lo: float = -2.0, origin_hi: float = 2.0, tmax: float = math.inf):
    """SoA rays: origins uniform in [lo, hi]^3, directions uniform on the sphere."""
    rs = Stream(seed, 2)
    o = rs.uniform(3 * n, origin_lo, origin_hi).reshape(n, 3).astype(np.float32)
    d = rs.unit_vectors(n).astype(np.float32)
    return dict(ox=np.ascontiguousarray(o[:, 0]), oy=np.ascontiguousarray(o[:, 1]),
                oz=np.ascontiguousarray(o[:, 2]), dx=np.ascontiguousarray(d[:, 0]),
                dy=np.ascontiguousarray(d[:, 1]), dz=np.ascontiguousarray(d[:, 2]),
                tmax=np.full(n, tmax, dtype=np.float32))


# --------------------------------------------------------------------------
# Workload 2: enclosed room for the path tracer
# --------------------------------------------------------------------------
def _grid_quad(origin, eu, ev, n: int, uv: bool = False):
    """A planar quad origin + [0,1]eu + [0,1]ev split into n x n cells (2 n^2
    triangles). Winding makes the normal cross(eu, ev). With uv, a fourth
    value: texcoords (u, v) = 2 (i, j) / n - 0.25, so a texture repeats about
    twice across the quad and wraps through negative coordinates."""
    i, j = np.meshgrid(np.arange(n + 1), np.arange(n + 1), indexing="ij")
    if uv:
        return _grid_quad(origin, eu, ev, n) + (np.stack([2 * i / n - 0.25, 2 * j / n - 0.25], -1).reshape(-1, 2),)
    v = (np.asarray(origin, np.float64)[None, None] + (i / n)[..., None] * np.asarray(eu, np.float64)
         + (j / n)[..., None] * np.asarray(ev, np.float64)).reshape(-1, 3)
    a = (np.arange(n)[:, None] * (n + 1) + np.arange(n)[None, :]).reshape(-1)
    f = np.concatenate([np.stack([a, a + n + 1, a + n + 2], 1), np.stack([a, a + n + 2, a + 1], 1)])
    nrm = np.cross(eu, ev)
    nrm = nrm / np.linalg.norm(nrm)
    return v, f, np.repeat(nrm[None], v.shape[0], 0)


CORNELL_CAMERA = ((0.0, 1.0, 3.4), (0.0, 1.0, 0.0), (0.0, 1.0, 0.0), 40.0)


def cornell_room(seed: int = 1, sphere_level: int = 6, wall_grid: int = 40, light_radiance: float = 10.0,
                 textured: bool = False):
    """Room [-1,1] x [0,2] x [-1,1] open towards +z: five wall quads (split
    into wall_grid^2 cells), two boxes rotated about y, an icosphere
    (level 6: 81,920 triangles) and a 0.5 x 0.5 ceiling light of radiance
    (10, 10, 10) facing down. Lambertian albedos uniform in [0.1, 0.9]^3.
    Defaults give about 100k triangles. Camera: CORNELL_CAMERA.

    textured: walls and light get texcoords (_grid_quad's uv) and the scene
    three RGBA textures ("textures", "material_textures" keys, the
    arguments of DeviceScene.set_textures): a 6 x 4 diffuse map on the
    floor, back and left walls, a 3 x 5 reflectiveness map (specular in
    [0, 0.3], exponent in [5, 60]) on the back wall and a 2 x 2 emissivity
    map in [5, 15] on the light."""
    rs = Stream(seed, 5)
    parts_v, parts_f, parts_n, parts_t, mat_ids, mats = [], [], [], [], [], []

    def add(v, f, n, mid, tc=None):
        base = sum(p.shape[0] for p in parts_v)
        parts_v.append(np.asarray(v, np.float64))
        parts_f.append(np.asarray(f) + base)
        parts_n.append(np.asarray(n, np.float64))
        parts_t.append(np.zeros((len(v), 2)) if tc is None else np.asarray(tc, np.float64))
        mat_ids.append(np.full(len(f), mid, np.uint32))

    def new_material(rec):
        mats.append(rec)
        return len(mats) - 1

    def albedo():
        return tuple(rs.uniform(3, 0.1, 0.9))

    g = wall_grid
    # (origin, eu, ev) with cross(eu, ev) pointing into the room
    walls = [((-1, 0, -1), (0, 0, 2), (2, 0, 0)),    # floor, normal +y
             ((-1, 2, -1), (2, 0, 0), (0, 0, 2)),    # ceiling, normal -y
             ((-1, 0, -1), (2, 0, 0), (0, 2, 0)),    # back wall z=-1, normal +z
             ((-1, 0, -1), (0, 2, 0), (0, 0, 2)),    # left wall x=-1, normal +x
             ((1, 0, -1), (0, 0, 2), (0, 2, 0))]     # right wall x=1, normal -x
    for o, eu, ev in walls:
        v, f, n, tc = _grid_quad(o, eu, ev, g, uv=True)
        add(v, f, n, new_material(lambert(albedo())), tc if textured else None)
    for center, half, angle in (((-0.35, 0.6, -0.3), (0.3, 0.6, 0.3), 0.3), ((0.4, 0.3, 0.3), (0.3, 0.3, 0.3), -0.3)):
        c, s = math.cos(angle), math.sin(angle)
        rot = np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]])
        mid = new_material(lambert(albedo()))
        for axis in range(3):
            for sign in (-1.0, 1.0):
                nrm = np.zeros(3)
                nrm[axis] = sign
                ua, va = [a for a in range(3) if a != axis]
                eu = np.zeros(3)
                ev = np.zeros(3)
                eu[ua] = 2 * half[ua]
                ev[va] = 2 * half[va]
                if np.dot(np.cross(eu, ev), nrm) < 0:
                    eu, ev = ev, eu
                o = np.zeros(3)
                o[axis] = sign * half[axis]
                o -= (eu + ev) / 2
                v, f, n = _grid_quad(o, eu, ev, 1)
                add(v @ rot.T + np.asarray(center), f, n @ rot.T, mid)
    sv, sf = icosphere(sphere_level)
    add(sv * 0.25 + np.array([0.45, 0.85, 0.3]), sf, sv, new_material(lambert(albedo())))
    lv, lf, ln, lt = _grid_quad((-0.25, 1.999, -0.25), (0.5, 0, 0), (0, 0, 0.5), 1, uv=True)  # normal -y
    add(lv, lf, ln, new_material(material_record(albedo=(0.0, 0.0, 0.0), specular=(0.0, 0.0, 0.0),
                                                 emissivity=(light_radiance,) * 3)), lt if textured else None)
    v = np.concatenate(parts_v)
    f = np.concatenate(parts_f)
    n = np.concatenate(parts_n)
    out = _pack(v, f, np.stack(mats), material_ids=np.concatenate(mat_ids), normals=n,
                texcoords=np.concatenate(parts_t))
    if textured:
        ts = Stream(seed, 6)
        diffuse = np.concatenate([ts.uniform(24, 0.1, 0.9).reshape(4, 6, 1).repeat(3, 2),
                                  np.ones((4, 6, 1))], 2)
        diffuse[..., 1] *= ts.uniform(24, 0.5, 1.0).reshape(4, 6)
        refl = np.concatenate([ts.uniform(45, 0.0, 0.3).reshape(5, 3, 3), ts.uniform(15, 5.0, 60.0).reshape(5, 3, 1)], 2)
        emis = np.concatenate([ts.uniform(4, 5.0, 15.0).reshape(2, 2, 1).repeat(3, 2), np.ones((2, 2, 1))], 2)
        mt = np.full((len(mats), 4), -1, np.int32)
        mt[[0, 2, 3], 2] = 0      # floor, back wall, left wall: diffuse map
        mt[2, 0] = 1              # back wall: reflectiveness map
        mt[len(mats) - 1, 3] = 2  # light: emissivity map
        out["textures"] = [t.astype(np.float32) for t in (diffuse, refl, emis)]
        out["material_textures"] = mt
    return out


def _value_noise(rs: Stream, n: int, cells: int) -> np.ndarray:
    """Bilinearly interpolated lattice noise in [-1, 1] on an n x n grid over [0, 1]^2."""
    lattice = rs.uniform((cells + 1) * (cells + 1), -1.0, 1.0).reshape(cells + 1, cells + 1)
    t = np.linspace(0.0, cells, n)
    i = np.minimum(t.astype(np.int64), cells - 1)
    f = t - i
    f = f * f * (3.0 - 2.0 * f)  # smoothstep fade
    a = lattice[i][:, i]
    b = lattice[i][:, i + 1]
    c = lattice[i + 1][:, i]
    d = lattice[i + 1][:, i + 1]
    fx, fz = f[:, None], f[None, :]
    return (a * (1 - fz) + b * fz) * (1 - fx) + (c * (1 - fz) + d * fz) * fx


def _flat_box(half: float):
    """Axis-aligned cube of half-size `half` about the origin: 6 faces of 4
    own vertices (flat shading normals), 12 outward triangles."""
    vs, fs, ns = [], [], []
    for axis in range(3):
        for sign in (-1.0, 1.0):
            nrm = np.zeros(3)
            nrm[axis] = sign
            ua, va = [a for a in range(3) if a != axis]
            eu = np.zeros(3)
            ev = np.zeros(3)
            eu[ua] = 2 * half
            ev[va] = 2 * half
            if np.dot(np.cross(eu, ev), nrm) < 0:
                eu, ev = ev, eu
            o = nrm * half - (eu + ev) / 2
            v, f, n = _grid_quad(o, eu, ev, 1)
            fs.append(f + 4 * len(vs))
            vs.append(v)
            ns.append(n)
    return np.concatenate(vs), np.concatenate(fs), np.concatenate(ns)


HEIGHTFIELD_CAMERA = ((0.0, 0.55, 1.35), (0.0, 0.0, -0.1), (0.0, 1.0, 0.0), 50.0)
HEIGHTFIELD_SUN = (0.45, 0.8, 0.4)   # towards the sun (normalised by the library)


def heightfield_boxes(seed: int = 1, grid: int = 512, amplitude: float = 0.2, num_boxes: int = 500,
                      octaves: int = 6):
    """The radiance-cache workload: a grid x grid-vertex fBm heightfield over
    [-1, 1]^2 (2 (grid-1)^2 triangles: 522,242 for 512) with heights scaled
    to +-amplitude, plus num_boxes boxes (side U[0.02, 0.08], rotated about
    y) standing on it. Lambertian albedos U[0.1, 0.8]^3: one material for the
    terrain, one per box. Lit by a directional sun (HEIGHTFIELD_SUN,
    irradiance 5) and a constant sky of 0.5 (renderer parameters).
    Camera: HEIGHTFIELD_CAMERA."""
    rs = Stream(seed, 11)
    h = np.zeros((grid, grid))
    amp, cells = 1.0, 4
    for _ in range(octaves):
        h += amp * _value_noise(rs, grid, cells)
        amp *= 0.5
        cells *= 2
    h *= amplitude / max(np.abs(h).max(), 1e-9)
    xs = np.linspace(-1.0, 1.0, grid)
    X, Z = np.meshgrid(xs, xs, indexing="ij")
    tv = np.stack([X, h, Z], -1).reshape(-1, 3)
    a = (np.arange(grid - 1)[:, None] * grid + np.arange(grid - 1)[None, :]).reshape(-1)
    # winding with +y normals: (a, a+1, a+grid+1), (a, a+grid+1, a+grid)
    tf = np.concatenate([np.stack([a, a + 1, a + grid + 1], 1), np.stack([a, a + grid + 1, a + grid], 1)])
    tn = vertex_normals(tv, tf)
    if tn[:, 1].mean() < 0:
        tf = tf[:, ::-1].copy()
        tn = -tn
    parts_v, parts_f, parts_n, ids = [tv], [tf], [tn], [np.zeros(len(tf), np.uint32)]
    mats = [lambert(tuple(rs.uniform(3, 0.1, 0.8)))]
    base = tv.shape[0]
    pos = rs.uniform(2 * num_boxes, -0.9, 0.9).reshape(num_boxes, 2)
    side = rs.uniform(num_boxes, 0.02, 0.08)
    ang = rs.uniform(num_boxes, 0.0, 2 * math.pi)
    for k in range(num_boxes):
        gi = int(round((pos[k, 0] + 1.0) * 0.5 * (grid - 1)))
        gk = int(round((pos[k, 1] + 1.0) * 0.5 * (grid - 1)))
        y0 = h[gi, gk]
        c, s = math.cos(ang[k]), math.sin(ang[k])
        rot = np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]])
        v, f, n = _flat_box(side[k] * 0.5)
        v = v @ rot.T + np.array([pos[k, 0], y0 + 0.4 * side[k], pos[k, 1]])
        parts_v.append(v)
        parts_f.append(f + base)
        parts_n.append(n @ rot.T)
        ids.append(np.full(len(f), len(mats), np.uint32))
        mats.append(lambert(tuple(rs.uniform(3, 0.1, 0.8))))
        base += v.shape[0]
    return _pack(np.concatenate(parts_v), np.concatenate(parts_f), np.stack(mats), material_ids=np.concatenate(ids),
                 normals=np.concatenate(parts_n))


def instanced_scene(seed: int = 1, num_triangles: int = 100_000, extent: float = 2.0):
    """Random instances of an icosphere (level 3), a box and a torus (scale
    U[0.05, 0.5], random rotation, position uniform in [-extent, extent]^3)
    flattened into one mesh until about num_triangles triangles, plus a
    ground quad below them and one area light (a random quad above the
    instances, radiance U[5, 20]). Lambertian albedos U[0.1, 0.9]^3, one of 16
    materials per instance. The batched-rendering workload draws 8 of these
    with log-uniform triangle counts."""
    rs = Stream(seed, 17)
    iv, iff = icosphere(3)
    bv, bf, bn = _flat_box(0.5)
    tv, tf = torus_mesh()
    meshes = [(iv, iff, iv), (bv, bf, bn), (tv, tf, vertex_normals(tv, tf))]
    mats = [lambert(tuple(rs.uniform(3, 0.1, 0.9))) for _ in range(16)]
    parts_v, parts_f, parts_n, ids = [], [], [], []
    base = 0
    total = 0
    while total < num_triangles:
        kind = int(rs.u64(1)[0] % 3)
        v0, f0, n0 = meshes[kind]
        s = rs.uniform(1, 0.05, 0.5)[0]
        rot = quat_to_matrix(rs.quaternions(1)[0])
        pos = rs.uniform(3, -extent, extent)
        parts_v.append((v0 * s) @ rot.T + pos)
        parts_n.append(n0 @ rot.T)
        parts_f.append(f0 + base)
        ids.append(np.full(len(f0), int(rs.u64(1)[0] % 16), np.uint32))
        base += v0.shape[0]
        total += len(f0)
    g = 1.5 * extent
    gv, gf, gn = _grid_quad((-g, -extent - 0.5, g), (2 * g, 0, 0), (0, 0, -2 * g), 1)  # ground, normal +y
    parts_v.append(gv)
    parts_f.append(gf + base)
    parts_n.append(gn)
    ids.append(np.full(len(gf), 0, np.uint32))
    base += gv.shape[0]
    size = rs.uniform(1, 0.5, 1.0)[0]
    lc = rs.uniform(2, -0.5 * extent, 0.5 * extent)
    lv, lf, ln = _grid_quad((lc[0] - size / 2, extent + 0.5, lc[1] - size / 2), (size, 0, 0), (0, 0, size), 1)
    radiance = rs.uniform(1, 5.0, 20.0)[0]
    mats.append(material_record(albedo=(0.0, 0.0, 0.0), specular=(0.0, 0.0, 0.0), emissivity=(radiance,) * 3))
    parts_v.append(lv)
    parts_f.append(lf + base)
    parts_n.append(ln)
    ids.append(np.full(len(lf), len(mats) - 1, np.uint32))
    return _pack(np.concatenate(parts_v), np.concatenate(parts_f), np.stack(mats), material_ids=np.concatenate(ids),
                 normals=np.concatenate(parts_n))


def large_instanced(seed: int = 1, num_instances: int = 20_000, volume: float = 100.0, num_lights: int = 256,
                    num_materials: int = 64):
    """The large BDPT workload: num_instances instances of a radially
    displaced icosphere (level 3, 1,280 triangles; 30 %) or a box (70 %),
    scale U[0.5, 2], random rotation, positions uniform in [0, volume]^3
    (about 7.9M triangles for 20k instances); num_materials materials, half
    Lambertian (albedo U[0.1, 0.9]^3), half Phong (specular U[0.2, 0.9]^3,
    exponent U[10, 1000]); num_lights light quads of side 0.5 with radiance
    log-uniform in [1, 100], facing random directions. Meant for an
    ellipsoid-bounded hierarchy."""
    rs = Stream(seed, 29)
    iv, iff = icosphere(3)
    disp = 1.0 + rs.uniform(iv.shape[0], -0.05, 0.05)
    iv = iv * disp[:, None]
    inrm = vertex_normals(iv, iff)
    bv, bf, bn = _flat_box(0.5)
    mats = []
    for k in range(num_materials):
        if k % 2 == 0:
            mats.append(lambert(tuple(rs.uniform(3, 0.1, 0.9))))
        else:
            exponent = rs.uniform(1, 10.0, 1000.0)[0]
            mats.append(material_record(albedo=tuple(rs.uniform(3, 0.05, 0.4)), specular=tuple(rs.uniform(3, 0.2, 0.9)),
                                        roughness=float(1.0 / math.sqrt(exponent))))
    kinds = (rs.u64(num_instances) % np.uint64(10)) < np.uint64(3)
    scale = rs.uniform(num_instances, 0.5, 2.0)
    quats = rs.quaternions(num_instances)
    pos = rs.uniform(3 * num_instances, 0.0, volume).reshape(num_instances, 3)
    matid = (rs.u64(num_instances) % np.uint64(num_materials)).astype(np.uint32)
    parts_v, parts_f, parts_n, ids = [], [], [], []
    base = 0
    for is_sphere, mesh in ((True, (iv, iff, inrm)), (False, (bv, bf, bn))):
        sel = np.nonzero(kinds == is_sphere)[0]
        v0, f0, n0 = mesh
        R = np.stack([quat_to_matrix(q) for q in quats[sel]])            # (k, 3, 3)
        vv = np.einsum("kij,vj->kvi", R, v0) * scale[sel][:, None, None] + pos[sel][:, None, :]
        nn = np.einsum("kij,vj->kvi", R, n0)
        ff = f0[None, :, :] + (base + np.arange(len(sel)) * v0.shape[0])[:, None, None]
        parts_v.append(vv.reshape(-1, 3))
        parts_n.append(nn.reshape(-1, 3))
        parts_f.append(ff.reshape(-1, 3))
        ids.append(np.repeat(matid[sel], f0.shape[0]))
        base += len(sel) * v0.shape[0]
    # lights: quads of side 0.5 with a random orientation
    lpos = rs.uniform(3 * num_lights, 0.0, volume).reshape(num_lights, 3)
    ldir = rs.unit_vectors(num_lights)
    lrad = np.exp(rs.uniform(num_lights, 0.0, math.log(100.0)))
    for k in range(num_lights):
        nrm = ldir[k]
        a = np.cross(nrm, [0.0, 1.0, 0.0] if abs(nrm[1]) < 0.9 else [1.0, 0.0, 0.0])
        a /= np.linalg.norm(a)
        b = np.cross(nrm, a)        # (b, a) winding makes the normal nrm: cross(b, a) = nrm
        v, f, n = _grid_quad(lpos[k] - 0.25 * (a + b), 0.5 * b, 0.5 * a, 1)
        parts_v.append(v)
        parts_f.append(f + base)
        parts_n.append(n)
        mats.append(material_record(albedo=(0.0, 0.0, 0.0), specular=(0.0, 0.0, 0.0), emissivity=(lrad[k],) * 3))
        ids.append(np.full(len(f), len(mats) - 1, np.uint32))
        base += v.shape[0]
    return _pack(np.concatenate(parts_v), np.concatenate(parts_f), np.stack(mats), material_ids=np.concatenate(ids),
                 normals=np.concatenate(parts_n))


LARGE_CAMERA = ((50.0, 50.0, -60.0), (50.0, 50.0, 50.0), (0.0, 1.0, 0.0), 55.0)
