"""ORACLE — test infrastructure only.

ctypes front end of oracle/_ref/libgpugi_ref.so: the reference's own shader
text (traceray.glsl, intersectiontests.glsl, random.glsl, helper.glsl and
pathtracer.comp with everything it includes) compiled as C++ by
oracle/ref_build.py. Used only by tests/ to pin the oracle's restatement.
available() is False where the reference tree is absent and no build was
made (the library is rebuilt from the tree, never stored in the repository).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import ref_build

_LIB = None


def available() -> bool:
    try:
        lib()
    except (OSError, RuntimeError):
        return False
    return True


def lib():
    global _LIB
    if _LIB is None:
        path = ref_build.build()
        if path is None or not path.exists():
            raise OSError("oracle/_ref is not built (the reference tree is absent)")
        L = C.CDLL(str(path))
        P, I, U32, U64 = C.c_void_p, C.c_int, C.c_uint32, C.c_uint64
        L.ref_trace_closest.argtypes = [P, P, P, I, I] + [P] * 7 + [U64, P, P, P, P, I]
        L.ref_trace_any.argtypes = [P, P, P, I, I] + [P] * 7 + [U64, P, I]
        L.ref_eval.argtypes = [I, U64, P, P]
        L.ref_render_pt.argtypes = [P, P, P, P, P, I, I, I, I, P, U32, P, I, P, P, I]
        for f in (L.ref_trace_closest, L.ref_trace_any, L.ref_eval, L.ref_render_pt):
            f.restype = I
        _LIB = L
    return _LIB


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _threads():
    return int(os.environ.get("ORACLE_THREADS", "0"))


def _rays(rays):
    return [np.ascontiguousarray(rays[k], dtype=np.float32) for k in ("ox", "oy", "oz", "dx", "dy", "dz", "tmax")]


def trace_closest(bvh, positions, rays) -> dict:
    """TraceRay of the reference: the hit Triangle record ({v0, v1, v2,
    material}, -1 on a miss), t, u = barycentric.y, v = barycentric.z."""
    hier = np.ascontiguousarray(bvh.hierarchy, dtype=np.float32)
    slots = np.ascontiguousarray(bvh.slots, dtype=np.int32)
    pos = np.ascontiguousarray(positions, dtype=np.float32)
    r = _rays(rays)
    n = r[0].shape[0]
    tri = np.empty((n, 4), np.int32)
    t, u, v = (np.empty(n, np.float32) for _ in range(3))
    rc = lib().ref_trace_closest(_p(hier), _p(slots), _p(pos), bvh.leaf_size, bvh.bounds_kind, *[_p(a) for a in r], n,
                                 _p(tri), _p(t), _p(u), _p(v), _threads())
    assert rc == 0, "AABB trees with leaf size 8 or 2, or oriented-box trees with leaf size 8"
    return dict(triangle=tri, t=t, u=u, v=v)


def trace_any(bvh, positions, rays) -> np.ndarray:
    hier = np.ascontiguousarray(bvh.hierarchy, dtype=np.float32)
    slots = np.ascontiguousarray(bvh.slots, dtype=np.int32)
    pos = np.ascontiguousarray(positions, dtype=np.float32)
    r = _rays(rays)
    n = r[0].shape[0]
    occ = np.empty(n, np.uint8)
    rc = lib().ref_trace_any(_p(hier), _p(slots), _p(pos), bvh.leaf_size, bvh.bounds_kind, *[_p(a) for a in r], n,
                             _p(occ), _threads())
    assert rc == 0, "AABB trees with leaf size 8 or 2, or oriented-box trees with leaf size 8"
    return occ


# kind: (input words per item, output words per item, output dtype)
EVAL_KINDS = {"wanghash": (0, 1, 1, np.uint32), "random_uint": (1, 1, 4, np.uint32), "random": (2, 1, 4, np.float32),
              "init_random_seed": (3, 2, 1, np.uint32), "sample_direction": (4, 2, 3, np.float32),
              "sample_hemisphere_cosine": (5, 5, 3, np.float32), "sample_phong_lobe": (6, 6, 3, np.float32),
              "create_onb": (7, 3, 6, np.float32), "unpack_normal": (8, 2, 3, np.float32),
              "pack_normal": (9, 3, 2, np.float32), "luminance": (10, 3, 1, np.float32)}


def _eval(fn, kind: str, inputs: np.ndarray) -> np.ndarray:
    k, win, wout, dt = EVAL_KINDS[kind]
    a = np.ascontiguousarray(inputs).reshape(-1, win)
    out = np.zeros((a.shape[0], wout), dt)
    assert fn(k, a.shape[0], _p(a), _p(out)) == 0
    return out


def evaluate(kind: str, inputs: np.ndarray) -> np.ndarray:
    """A random.glsl / helper.glsl function of the reference over rows of inputs."""
    return _eval(lib().ref_eval, kind, inputs)


def evaluate_oracle(kind: str, inputs: np.ndarray) -> np.ndarray:
    """The oracle's restatement of the same function (reference streams)."""
    from . import lib as olib
    L = olib()
    L.oracle_eval.argtypes = [C.c_int, C.c_uint64, C.c_void_p, C.c_void_p]
    L.oracle_eval.restype = C.c_int
    return _eval(L.oracle_eval, kind, inputs)


def render_pt(bvh, scene: dict, width: int, height: int, camera: np.ndarray, frame_seed: int,
              light_samples: np.ndarray, max_path_length: int = 8, sky=(0.0, 0.0, 0.0),
              accum: np.ndarray | None = None) -> np.ndarray:
    """One iteration of the reference's pathtracer.comp over every pixel,
    accumulated into accum (H, W, 4) float32."""
    from gpugi_gb300.cuda import vertex_info  # host-side layout helper (no compute)
    assert bvh.leaf_size == 8 and bvh.bounds_kind == 0, "the path tracer is built for 8-slot AABB hierarchies"
    hier = np.ascontiguousarray(bvh.hierarchy, dtype=np.float32)
    slots = np.ascontiguousarray(bvh.slots, dtype=np.int32)
    pos = np.ascontiguousarray(scene["positions"], dtype=np.float32)
    vi = np.ascontiguousarray(vertex_info(scene["normals"], scene["texcoords"]), dtype=np.float32)
    mats = np.ascontiguousarray(scene["materials"], dtype=np.float32).reshape(-1, 24)
    cam = np.ascontiguousarray(camera, dtype=np.float32)
    ls = np.ascontiguousarray(light_samples, dtype=np.float32).reshape(-1, 8)
    skya = np.asarray(sky, dtype=np.float32)
    if accum is None:
        accum = np.zeros((height, width, 4), np.float32)
    assert accum.dtype == np.float32 and accum.flags.c_contiguous
    rc = lib().ref_render_pt(_p(hier), _p(slots), _p(pos), _p(vi), _p(mats), mats.shape[0], width, height,
                             max_path_length, _p(cam), frame_seed & 0xFFFFFFFF, _p(ls), ls.shape[0], _p(skya),
                             _p(accum), _threads())
    assert rc == 0
    return accum


def render_lt(bvh, scene: dict, width: int, height: int, camera: np.ndarray, frame_seed: int,
              light_samples: np.ndarray, max_path_length: int = 8, accum: np.ndarray | None = None,
              bidir: bool = False, rays_per_light_sample: int | None = None, param: float = 0.0,
              position: np.ndarray | None = None) -> np.ndarray:
    """One iteration of LightPathtracer::Draw with the reference's
    lighttracer.comp and showlightcaches.comp, or (bidir) of
    BidirectionalPathtracer::Draw with lighttracer.comp (SAVE_LIGHT_CACHE)
    and pathtracer_bidir.comp; invocations in order on one thread,
    accumulated into accum (H, W, 4) float32. Rays per light sample as
    LightPathtracer::SetScreenSize (lightpathtracer.cpp:34)."""
    from gpugi_gb300.cuda import vertex_info  # host-side layout helper (no compute)
    assert bvh.leaf_size == 8 and bvh.bounds_kind == 0, "the light tracer is built for 8-slot AABB hierarchies"
    L = lib()
    L.ref_render_lt.argtypes = [C.c_void_p] * 5 + [C.c_int] * 4 + [C.c_void_p, C.c_uint32, C.c_void_p, C.c_int,
                                                                    C.c_int, C.c_int, C.c_float, C.c_void_p,
                                                                    C.c_void_p]
    L.ref_render_lt.restype = C.c_int
    hier = np.ascontiguousarray(bvh.hierarchy, dtype=np.float32)
    slots = np.ascontiguousarray(bvh.slots, dtype=np.int32)
    pos = np.ascontiguousarray(scene["positions"], dtype=np.float32)
    vi = np.ascontiguousarray(vertex_info(scene["normals"], scene["texcoords"]), dtype=np.float32)
    mats = np.ascontiguousarray(scene["materials"], dtype=np.float32).reshape(-1, 24)
    cam = np.ascontiguousarray(camera, dtype=np.float32)
    ls = np.ascontiguousarray(light_samples, dtype=np.float32).reshape(-1, 8)
    rays = rays_per_light_sample or max(64, (width * height // ls.shape[0] // 64) * 64)
    if accum is None:
        accum = np.zeros((height, width, 4), np.float32)
    assert accum.dtype == np.float32 and accum.flags.c_contiguous
    rc = L.ref_render_lt(_p(hier), _p(slots), _p(pos), _p(vi), _p(mats), mats.shape[0], width, height,
                         max_path_length, _p(cam), frame_seed & 0xFFFFFFFF, _p(ls), ls.shape[0], rays, int(bidir),
                         float(param), _p(accum), None if position is None else _p(position))
    assert rc == 0
    return accum


def _render_light(bvh, scene, width, height, camera, frame_seed, light_samples, max_path_length, accum, kind):
    return render_lt(bvh, scene, width, height, camera, frame_seed, light_samples, max_path_length, accum, kind)


def render_whitted(bvh, scene: dict, width: int, height: int, camera: np.ndarray, frame_seed: int,
                   light_samples: np.ndarray, max_path_length: int = 8, accum: np.ndarray | None = None) -> np.ndarray:
    """One iteration of WhittedRayTracer::Draw with the reference's
    whittedraytracer.comp (STOP_ON_DIFFUSE_BOUNCE, whittedraytracer.cpp:40),
    pixels in order on one thread, accumulated into accum (H, W, 4)."""
    return _render_light(bvh, scene, width, height, camera, frame_seed, light_samples, max_path_length, accum, 2)


def render_pm(bvh, scene: dict, width: int, height: int, camera: np.ndarray, frame_seed: int,
              light_samples: np.ndarray, max_path_length: int = 8, accum: np.ndarray | None = None,
              photons_per_light_sample: int = 2048, query_radius: float = 0.01) -> np.ndarray:
    """One iteration of PhotonMapper::Draw with the reference's
    photondistribution.comp and gather.comp (lossless hash map,
    maps/hashmap.glsl), invocations in order on one thread."""
    return render_lt(bvh, scene, width, height, camera, frame_seed, light_samples, max_path_length, accum, 3,
                     rays_per_light_sample=photons_per_light_sample, param=query_radius)


def render_im(bvh, scene: dict, width: int, height: int, camera: np.ndarray, frame_seed: int,
              light_samples: np.ndarray, accum: np.ndarray, position: np.ndarray, max_path_length: int = 8,
              photons_per_light_sample: int = 2048, query_radius: float = 0.005) -> np.ndarray:
    """One iteration of PixelMapLighttracer::Draw with the reference's
    importondistribution.comp and photontracing.comp (DEPTH_BUFFER_OCCLUSION_TEST,
    lossless hash map), invocations in order on one thread. accum (H, W, 4)
    holds the reference's image (alpha: the first hit's packed normal x),
    position (H, W, 4) its position texture; both carry over iterations."""
    assert position.dtype == np.float32 and position.shape == (height, width, 4) and position.flags.c_contiguous
    return render_lt(bvh, scene, width, height, camera, frame_seed, light_samples, max_path_length, accum, 4,
                     rays_per_light_sample=photons_per_light_sample, param=query_radius, position=position)



def render_hier(bvh, scene: dict, width: int, height: int, camera: np.ndarray, frame_seed: int,
                light_samples: np.ndarray, importance: np.ndarray, materials: np.ndarray, sggx: np.ndarray,
                sky=(0.0, 0.0, 0.0), accum: np.ndarray | None = None) -> np.ndarray:
    """One iteration of HierarchyImportance's renderer with the reference's
    hierarchypathtracer.comp (its own MAX_PATHLENGTH 4), pixels in order on
    one thread, accumulated into accum (H, W, 4) float32. importance: (nodes
    + slots, 2) float32; materials: the node materials as packed halves
    (uint32, six RGBA16F texels per node); sggx: (nodes, 6) uint16."""
    from gpugi_gb300.cuda import vertex_info  # host-side layout helper (no compute)
    assert bvh.leaf_size == 8 and bvh.bounds_kind == 0, "the path tracer is built for 8-slot AABB hierarchies"
    L = lib()
    P, I, U64 = C.c_void_p, C.c_int, C.c_uint64
    L.ref_render_hier.argtypes = [P] * 5 + [I, I, I, P, C.c_uint32, P, I, P, P, P, U64, P, U64, P]
    L.ref_render_hier.restype = I
    hier = np.ascontiguousarray(bvh.hierarchy, dtype=np.float32)
    slots = np.ascontiguousarray(bvh.slots, dtype=np.int32)
    pos = np.ascontiguousarray(scene["positions"], dtype=np.float32)
    vi = np.ascontiguousarray(vertex_info(scene["normals"], scene["texcoords"]), dtype=np.float32)
    mats = np.ascontiguousarray(scene["materials"], dtype=np.float32).reshape(-1, 24)
    cam = np.ascontiguousarray(camera, dtype=np.float32)
    ls = np.ascontiguousarray(light_samples, dtype=np.float32).reshape(-1, 8)
    imp = np.ascontiguousarray(importance, dtype=np.float32)
    hm = np.ascontiguousarray(materials, dtype=np.uint32).view(np.uint16).reshape(-1)
    sg = np.ascontiguousarray(sggx, dtype=np.uint16).reshape(-1)
    skya = np.asarray(sky, dtype=np.float32)
    if accum is None:
        accum = np.zeros((height, width, 4), np.float32)
    assert accum.dtype == np.float32 and accum.flags.c_contiguous
    rc = L.ref_render_hier(_p(hier), _p(slots), _p(pos), _p(vi), _p(mats), mats.shape[0], width, height, _p(cam),
                           frame_seed & 0xFFFFFFFF, _p(ls), ls.shape[0], _p(skya), _p(imp), _p(hm), hm.size, _p(sg),
                           sg.size, _p(accum))
    assert rc == 0
    return accum


def _hier_scene(bvh, scene):
    from gpugi_gb300.cuda import vertex_info  # host-side layout helper (no compute)
    assert bvh.leaf_size == 8 and bvh.bounds_kind == 0, "the hierarchy passes are built for 8-slot AABB hierarchies"
    return (np.ascontiguousarray(bvh.hierarchy, dtype=np.float32), np.ascontiguousarray(bvh.slots, dtype=np.int32),
            np.ascontiguousarray(scene["positions"], dtype=np.float32),
            np.ascontiguousarray(vertex_info(scene["normals"], scene["texcoords"]), dtype=np.float32),
            np.ascontiguousarray(scene["materials"], dtype=np.float32).reshape(-1, 24))


def hier_importance(bvh, scene: dict, width: int, height: int, camera: np.ndarray, light_samples: np.ndarray,
                    iterations: int = 10):
    """HierarchyImportance's importance pass with the reference's
    acquisition2.comp (NumImportanceIterations = 1..iterations), then
    hierarchypropagation_init.comp and hierarchypropagation_nodes.comp until
    nothing changes; invocations in order on one thread. Returns (importance
    float32 [nodes + slots, 2], subtree float32 [nodes])."""
    L = lib()
    P, I = C.c_void_p, C.c_int
    L.ref_hier_importance.argtypes = [P, I, P, I, P, P, P, I, I, I, P, P, I, I, P, P]
    L.ref_hier_importance.restype = I
    hier, slots, pos, vi, mats = _hier_scene(bvh, scene)
    cam = np.ascontiguousarray(camera, dtype=np.float32)
    ls = np.ascontiguousarray(light_samples, dtype=np.float32).reshape(-1, 8)
    imp = np.zeros((hier.shape[0] + slots.shape[0], 2), np.float32)
    sub = np.zeros(hier.shape[0], np.float32)
    rc = L.ref_hier_importance(_p(hier), hier.shape[0], _p(slots), slots.shape[0], _p(pos), _p(vi), _p(mats),
                               mats.shape[0], width, height, _p(cam), _p(ls), ls.shape[0], iterations, _p(imp),
                               _p(sub))
    assert rc == 0
    return imp, sub


def hier_materials(bvh, scene: dict) -> np.ndarray:
    """Node materials with the reference's sampleleafmaterials.comp, then
    pullmaterials.comp once per tree level: uint32 [nodes, 12], six pairs of
    packed halves per node."""
    L = lib()
    P, I = C.c_void_p, C.c_int
    L.ref_hier_materials.argtypes = [P, I, P, P, P, P, I, P]
    L.ref_hier_materials.restype = I
    hier, slots, pos, vi, mats = _hier_scene(bvh, scene)
    out = np.zeros((hier.shape[0], 12), np.uint32)
    rc = L.ref_hier_materials(_p(hier), hier.shape[0], _p(slots), _p(pos), _p(vi), _p(mats), mats.shape[0], _p(out))
    assert rc == 0
    return out
