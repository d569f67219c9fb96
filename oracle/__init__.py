"""ORACLE — test infrastructure only.

ctypes front end of oracle/lib/liboracle.so, the CPU restatement of gpugi's
shaders. Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline
leg may import this package; the product never does.

Parity status: UNPINNED (the reference ships no golden vectors and cannot be
built or run here); see oracle/glsl.hpp.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        from . import build as _b
        path = _b.build()
        L = C.CDLL(str(path))
        P, U32, U64, I = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int
        L.oracle_trace_closest.argtypes = [P, U32, U32, P, U32, U32, P, U32] + [P] * 7 + [U64, P, P, P, P, P, I]
        L.oracle_trace_any.argtypes = [P, U32, U32, P, U32, U32, P, U32] + [P] * 7 + [U64, P, P, I]
        L.oracle_bruteforce_closest.argtypes = [P, U32, P] + [P] * 7 + [U64, P, P, I]
        if hasattr(L, "oracle_render"):
            L.oracle_render.restype = I
        _LIB = L
    return _LIB


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def threads() -> int:
    return int(os.environ.get("ORACLE_THREADS", "0"))


def _scene_args(bvh, positions):
    hier = np.ascontiguousarray(bvh.hierarchy, dtype=np.float32)
    slots = np.ascontiguousarray(bvh.slots, dtype=np.int32)
    pos = np.ascontiguousarray(positions, dtype=np.float32)
    keep = (hier, slots, pos)
    return keep, [_p(hier), hier.shape[0], bvh.bounds_kind, _p(slots), slots.shape[0], bvh.leaf_size, _p(pos),
                  pos.shape[0]]


def _rays(rays):
    return [np.ascontiguousarray(rays[k], dtype=np.float32) for k in ("ox", "oy", "oz", "dx", "dy", "dz", "tmax")]


def set_triangle_test(watertight: bool) -> None:
    """Triangle test of the following query calls: the reference's
    IntersectTriangle or the watertight test."""
    L = lib()
    L.oracle_set_triangle_test.argtypes = [C.c_int]
    L.oracle_set_triangle_test.restype = None
    L.oracle_set_triangle_test(1 if watertight else 0)


def trace_closest(bvh, positions, rays, counters=False, num_threads=None, watertight=False):
    set_triangle_test(watertight)
    keep, sargs = _scene_args(bvh, positions)
    r = _rays(rays)
    n = r[0].shape[0]
    slot = np.empty(n, np.int32)
    t = np.empty(n, np.float32)
    u = np.empty(n, np.float32)
    v = np.empty(n, np.float32)
    cnt = np.empty((n, 3), np.uint32) if counters else None
    lib().oracle_trace_closest(*sargs, *[_p(a) for a in r], n, _p(slot), _p(t), _p(u), _p(v), _p(cnt),
                               threads() if num_threads is None else num_threads)
    out = dict(slot=slot, t=t, u=u, v=v)
    if counters:
        out["counters"] = cnt
    return out


def trace_any(bvh, positions, rays, counters=False, num_threads=None, watertight=False):
    set_triangle_test(watertight)
    keep, sargs = _scene_args(bvh, positions)
    r = _rays(rays)
    n = r[0].shape[0]
    occ = np.empty(n, np.uint8)
    cnt = np.empty((n, 3), np.uint32) if counters else None
    lib().oracle_trace_any(*sargs, *[_p(a) for a in r], n, _p(occ), _p(cnt),
                           threads() if num_threads is None else num_threads)
    out = dict(occluded=occ)
    if counters:
        out["counters"] = cnt
    return out


def bruteforce_closest(slots, positions, rays, num_threads=None, watertight=False):
    set_triangle_test(watertight)
    slots = np.ascontiguousarray(slots, dtype=np.int32)
    pos = np.ascontiguousarray(positions, dtype=np.float32)
    r = _rays(rays)
    n = r[0].shape[0]
    slot = np.empty(n, np.int32)
    t = np.empty(n, np.float32)
    lib().oracle_bruteforce_closest(_p(slots), slots.shape[0], _p(pos), *[_p(a) for a in r], n, _p(slot), _p(t),
                                    threads() if num_threads is None else num_threads)
    return dict(slot=slot, t=t)


PASSES = {"PT": 0, "LT": 1, "BPT": 2, "WHITTED": 3}


def render(bvh, scene: dict, pass_: str, width: int, height: int, camera: np.ndarray, frame_seed: int,
           light_samples: np.ndarray, max_path_length: int = 8, rr_start_depth: int = 0, sky=(0.0, 0.0, 0.0),
           accum: np.ndarray | None = None, num_threads=None, photons_per_light_sample: int = 2048,
           query_radius: float = 0.01, gbuffer: np.ndarray | None = None, rng: str = "pcg") -> np.ndarray:
    """One iteration of a pass (restated pathtracer.comp / lighttracer.comp /
    BPT / whittedraytracer.comp / the photon mapper "PM" / the importon map
    light tracer "IM"), accumulated into accum (H, W, 4) float32, which is
    returned. "IM" also needs gbuffer, an (H, W, 5) float32 array of the
    first eye hits that the caller carries from iteration to iteration
    (zeros before the first). rng: "pcg" or "reference" random streams;
    frame_seed must be that generator's FrameSeed of the iteration."""
    from gpugi_gb300.cuda import vertex_info  # host-side layout helper (no compute)
    L = lib()
    set_rng(rng)
    P, U32, I, F = C.c_void_p, C.c_uint32, C.c_int, C.c_float
    L.oracle_render.argtypes = [P, U32, U32, P, U32, U32, P, P, U32, P, U32, I, I, I, I, I, P, U32, P, I, P, P, I]
    hier = np.ascontiguousarray(bvh.hierarchy, dtype=np.float32)
    slots = np.ascontiguousarray(bvh.slots, dtype=np.int32)
    pos = np.ascontiguousarray(scene["positions"], dtype=np.float32)
    vi = np.ascontiguousarray(vertex_info(scene["normals"], scene["texcoords"]), dtype=np.float32)
    mats = np.ascontiguousarray(scene["materials"], dtype=np.float32)
    cam = np.ascontiguousarray(camera, dtype=np.float32)
    ls = np.ascontiguousarray(light_samples, dtype=np.float32).reshape(-1, 8)
    skya = np.asarray(sky, dtype=np.float32)
    if accum is None:
        accum = np.zeros((height, width, 4), np.float32)
    nt = threads() if num_threads is None else num_threads
    if pass_ == "PM":
        L.oracle_render_pm.argtypes = [P, U32, U32, P, U32, U32, P, P, U32, P, U32, I, I, I, I, P, U32, P, I, P, I,
                                       F, P, I]
        rc = L.oracle_render_pm(_p(hier), hier.shape[0], bvh.bounds_kind, _p(slots), slots.shape[0], bvh.leaf_size,
                                _p(pos), _p(vi), pos.shape[0], _p(mats), mats.shape[0], width, height,
                                max_path_length, rr_start_depth, _p(cam), frame_seed & 0xFFFFFFFF, _p(ls),
                                ls.shape[0], _p(skya), photons_per_light_sample, float(query_radius), _p(accum), nt)
        assert rc == 0
        return accum
    if pass_ == "IM":
        assert gbuffer is not None and gbuffer.shape == (height, width, 5) and gbuffer.dtype == np.float32
        assert gbuffer.flags.c_contiguous
        L.oracle_render_im.argtypes = [P, U32, U32, P, U32, U32, P, P, U32, P, U32, I, I, I, I, P, U32, P, I, P, I,
                                       F, P, P, I]
        rc = L.oracle_render_im(_p(hier), hier.shape[0], bvh.bounds_kind, _p(slots), slots.shape[0], bvh.leaf_size,
                                _p(pos), _p(vi), pos.shape[0], _p(mats), mats.shape[0], width, height,
                                max_path_length, rr_start_depth, _p(cam), frame_seed & 0xFFFFFFFF, _p(ls),
                                ls.shape[0], _p(skya), photons_per_light_sample, float(query_radius), _p(accum),
                                _p(gbuffer), nt)
        assert rc == 0
        return accum
    rc = L.oracle_render(_p(hier), hier.shape[0], bvh.bounds_kind, _p(slots), slots.shape[0], bvh.leaf_size,
                         _p(pos), _p(vi), pos.shape[0], _p(mats), mats.shape[0], PASSES[pass_], width, height,
                         max_path_length, rr_start_depth, _p(cam), frame_seed & 0xFFFFFFFF, _p(ls), ls.shape[0],
                         _p(skya), _p(accum), nt)
    assert rc == 0
    return accum


_TEXTURES = None


def set_textures(textures, material_textures) -> None:
    """Material textures of the following rendering calls, as
    DeviceScene.set_textures takes them; None or [] removes them."""
    global _TEXTURES
    L = lib()
    L.oracle_set_textures.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32]
    L.oracle_set_textures.restype = None
    if not textures:
        _TEXTURES = None
        L.oracle_set_textures(None, None, None, 0)
        return
    texels = np.ascontiguousarray(np.concatenate([np.asarray(t, np.float32).reshape(-1, 4) for t in textures]))
    info = np.zeros((len(textures), 4), np.uint32)
    at = 0
    for i, t in enumerate(textures):
        info[i] = (at, t.shape[1], t.shape[0], 0)
        at += t.shape[0] * t.shape[1]
    mt = np.ascontiguousarray(material_textures, dtype=np.int32).reshape(-1, 4)
    _TEXTURES = (texels, info, mt)
    L.oracle_set_textures(_p(texels), _p(info), _p(mt), mt.shape[0])


def set_rng(rng: str) -> None:
    """Random streams of the following rendering calls ("pcg" or "reference")."""
    if rng not in ("pcg", "reference"):
        raise ValueError(rng)
    L = lib()
    L.oracle_set_rng.argtypes = [C.c_int]
    L.oracle_set_rng.restype = None
    L.oracle_set_rng(1 if rng == "pcg" else 0)


def _render_scene_args(bvh, scene):
    from gpugi_gb300.cuda import vertex_info  # host-side layout helper (no compute)
    hier = np.ascontiguousarray(bvh.hierarchy, dtype=np.float32)
    slots = np.ascontiguousarray(bvh.slots, dtype=np.int32)
    pos = np.ascontiguousarray(scene["positions"], dtype=np.float32)
    vi = np.ascontiguousarray(vertex_info(scene["normals"], scene["texcoords"]), dtype=np.float32)
    mats = np.ascontiguousarray(scene["materials"], dtype=np.float32)
    keep = (hier, slots, pos, vi, mats)
    return keep, [_p(hier), hier.shape[0], _p(slots), slots.shape[0], bvh.leaf_size, _p(pos), _p(vi),
                  pos.shape[0], _p(mats), mats.shape[0]]


_SCENE_T = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p, C.c_uint32,
            C.c_void_p, C.c_uint32]


def hier_importance(bvh, scene: dict, width: int, height: int, camera: np.ndarray, light_samples: np.ndarray,
                    iterations: int = 10, num_threads=None):
    """HierarchyImportance's importance pass (acquisition2.comp x iterations,
    then the propagation) on an AABB hierarchy: returns (importance
    float32 [numNodes + numSlots, 2], subtree float32 [numNodes])."""
    assert bvh.bounds_kind == 0
    L = lib()
    I = C.c_int
    L.oracle_hier_importance.argtypes = _SCENE_T + [I, I, C.c_void_p, C.c_void_p, I, I, C.c_void_p, C.c_void_p, I]
    L.oracle_hier_importance.restype = I
    keep, sargs = _render_scene_args(bvh, scene)
    cam = np.ascontiguousarray(camera, dtype=np.float32)
    ls = np.ascontiguousarray(light_samples, dtype=np.float32).reshape(-1, 8)
    imp = np.zeros((bvh.num_nodes + bvh.num_slots, 2), np.float32)
    sub = np.zeros(bvh.num_nodes, np.float32)
    rc = L.oracle_hier_importance(*sargs, width, height, _p(cam), _p(ls), ls.shape[0], iterations, _p(imp), _p(sub),
                                  threads() if num_threads is None else num_threads)
    assert rc == 0
    return imp, sub


def hier_propagate(bvh, importance: np.ndarray, iterations: int):
    """The propagation alone: importance [numNodes + numSlots, 2] with the
    accumulated x; returns (importance with x / iterations and y, subtree)."""
    L = lib()
    L.oracle_hier_propagate.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_uint32, C.c_int,
                                        C.c_void_p, C.c_void_p]
    L.oracle_hier_propagate.restype = C.c_int
    hier = np.ascontiguousarray(bvh.hierarchy, dtype=np.float32)
    slots = np.ascontiguousarray(bvh.slots, dtype=np.int32)
    imp = np.array(importance, dtype=np.float32, copy=True, order="C")
    sub = np.zeros(bvh.num_nodes, np.float32)
    assert L.oracle_hier_propagate(_p(hier), hier.shape[0], _p(slots), slots.shape[0], bvh.leaf_size, iterations,
                                   _p(imp), _p(sub)) == 0
    return imp, sub


def hier_materials(bvh, scene: dict) -> np.ndarray:
    """Node materials (sampleleafmaterials.comp + pullmaterials.comp):
    uint32 [numNodes, 12], six pairs of packed halves per node."""
    L = lib()
    L.oracle_hier_materials.argtypes = _SCENE_T + [C.c_void_p]
    L.oracle_hier_materials.restype = C.c_int
    keep, sargs = _render_scene_args(bvh, scene)
    out = np.zeros((bvh.num_nodes, 12), np.uint32)
    assert L.oracle_hier_materials(*sargs, _p(out)) == 0
    return out


def render_hier(bvh, scene: dict, width: int, height: int, camera: np.ndarray, frame_seed: int,
                light_samples: np.ndarray, importance: np.ndarray, materials: np.ndarray, sggx: np.ndarray,
                max_path_length: int = 4, sky=(0.0, 0.0, 0.0), accum: np.ndarray | None = None,
                num_threads=None, rng: str = "pcg") -> np.ndarray:
    """One iteration of hierarchypathtracer.comp, accumulated into accum (H, W, 4)."""
    L = lib()
    set_rng(rng)
    I = C.c_int
    L.oracle_render_hier.argtypes = _SCENE_T + [I, I, I, C.c_void_p, C.c_uint32, C.c_void_p, I, C.c_void_p,
                                                C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, I]
    L.oracle_render_hier.restype = I
    keep, sargs = _render_scene_args(bvh, scene)
    cam = np.ascontiguousarray(camera, dtype=np.float32)
    ls = np.ascontiguousarray(light_samples, dtype=np.float32).reshape(-1, 8)
    imp = np.ascontiguousarray(importance, dtype=np.float32)
    mats = np.ascontiguousarray(materials, dtype=np.uint32)
    sg = np.ascontiguousarray(sggx, dtype=np.uint16)
    skya = np.asarray(sky, dtype=np.float32)
    if accum is None:
        accum = np.zeros((height, width, 4), np.float32)
    rc = L.oracle_render_hier(*sargs, width, height, max_path_length, _p(cam), frame_seed & 0xFFFFFFFF, _p(ls),
                              ls.shape[0], _p(skya), _p(imp), _p(mats), _p(sg), _p(accum),
                              threads() if num_threads is None else num_threads)
    assert rc == 0
    return accum


def light_samples(positions, slots, materials, num_samples: int, rng_state: list, point_lights=(),
                  directional_lights=()) -> np.ndarray:
    """LightSampler::GenerateRandomSamples (restated, lights.cpp) over a
    scene's triangle slots and materials; point_lights: (position,
    intensity) pairs, directional_lights: (unit direction towards the light,
    irradiance) pairs. rng_state: one-element list with the 64-bit xorshift*
    state, updated. Returns (num_samples, 8) float32."""
    L = lib()
    P, U32 = C.c_void_p, C.c_uint32
    L.oracle_light_samples.argtypes = [P, P, U32, P, P, U32, P, U32, C.POINTER(C.c_uint64), U32, P]
    L.oracle_light_samples.restype = C.c_int
    pos = np.ascontiguousarray(positions, dtype=np.float32)
    sl = np.ascontiguousarray(slots, dtype=np.int32).reshape(-1, 4)
    mats = np.ascontiguousarray(materials, dtype=np.float32).reshape(-1)
    pts = np.ascontiguousarray(np.array([list(p) + list(i) for p, i in point_lights], np.float32).reshape(-1, 6))
    drs = np.ascontiguousarray(np.array([list(d) + list(e) for d, e in directional_lights], np.float32).reshape(-1, 6))
    out = np.zeros((num_samples, 8), np.float32)
    st = C.c_uint64(rng_state[0])
    rc = L.oracle_light_samples(_p(pos), _p(sl), sl.shape[0], _p(mats), _p(pts), pts.shape[0], _p(drs), drs.shape[0],
                                C.byref(st), num_samples, _p(out))
    assert rc == 0, "light sample outside the summed table"
    rng_state[0] = st.value
    return out


def float_to_half(x: np.ndarray) -> np.ndarray:
    L = lib()
    L.oracle_float_to_half.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64]
    x = np.ascontiguousarray(x, dtype=np.float32)
    out = np.empty(x.shape, np.uint16)
    L.oracle_float_to_half(_p(x), _p(out), x.size)
    return out


def half_to_float(h: np.ndarray) -> np.ndarray:
    L = lib()
    L.oracle_half_to_float.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64]
    h = np.ascontiguousarray(h, dtype=np.uint16)
    out = np.empty(h.shape, np.float32)
    L.oracle_half_to_float(_p(h), _p(out), h.size)
    return out


def algorithmic_bytes(counters: np.ndarray, any_hit: bool = False) -> np.ndarray:
    """Bytes per ray of gpugi's own fetch pattern: 24 (ray in) + 16 (t, id, u, v
    out; 4 for any-hit) + 32 per node + 16 per leaf slot + 36 per valid triangle
    (node 32 B, gpugi/scene/scene.hpp:30-38; slot 16 B, traceray.glsl:126;
    3 x 12 B positions, traceray.glsl:137-139)."""
    c = counters.astype(np.int64)
    out_bytes = 4 if any_hit else 16
    return 24 + out_bytes + 32 * c[:, 0] + 16 * c[:, 1] + 36 * c[:, 2]
