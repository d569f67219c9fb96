"""ctypes front end of libgpugi_cuda.so (include/gpugi_cuda.h).

This module only binds the C ABI; it has no compute of its own and no CPU
fallback. Loading fails loudly when the library is missing.
"""
from __future__ import annotations

import atexit
import ctypes as C
import os
import weakref
from pathlib import Path

import numpy as np

LIB_DIR = Path(__file__).resolve().parent / "lib"
_LIB = None

STATUS = {0: "OK", 1: "INVALID_ARGUMENT", 2: "INVALID_SCENE", 3: "OUT_OF_MEMORY", 4: "CUDA", 5: "DEVICE",
          6: "UNSUPPORTED"}


class GpugiError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"gpugi status {status} ({STATUS.get(status, '?')}): {msg}")
        self.status = status


def lib():
    """The CUDA library: libgpugi_cuda.so, or with GPUGI_CHECKED=1 in the
    environment the bounds-checked libgpugi_cuda_checked.so."""
    global _LIB
    if _LIB is None:
        checked = os.environ.get("GPUGI_CHECKED", "0") not in ("", "0")
        path = LIB_DIR / ("libgpugi_cuda_checked.so" if checked else "libgpugi_cuda.so")
        if not path.exists():
            raise RuntimeError(f"{path} is missing: the CUDA extension must be built (python -m gpugi_gb300.build)")
        _LIB = C.CDLL(str(path))
        _declare(_LIB)
    return _LIB


def _declare(L):
    P, U32, U64, I, F = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int, C.c_float
    L.gpugi_create.argtypes = [C.POINTER(P), P]
    L.gpugi_destroy.argtypes = [P]
    L.gpugi_destroy.restype = None
    L.gpugi_last_error.argtypes = [P]
    L.gpugi_last_error.restype = C.c_char_p
    L.gpugi_sync.argtypes = [P]
    L.gpugi_device_error_bits.argtypes = [P, C.POINTER(U32)]
    L.gpugi_stream.argtypes = [P]
    L.gpugi_stream.restype = P
    L.gpugi_version.restype = C.c_char_p
    L.gpugi_scene_upload.argtypes = [P, P, U32, U32, P, U32, U32, P, P, U32, P, U32, C.POINTER(P)]
    L.gpugi_scene_destroy.argtypes = [P]
    L.gpugi_scene_destroy.restype = None
    L.gpugi_debug_raise_device_error.argtypes = [P, U32]
    L.gpugi_debug_limit_nodes.argtypes = [P, U32]
    L.gpugi_set_async_walker_share.argtypes = [P, U32]
    L.gpugi_nrc_debug_stall.argtypes = [P, P, U32, U64]
    L.gpugi_scene_build.argtypes = [P, P, U32, P, U32, P, P, U32, U32, C.POINTER(P)]
    L.gpugi_scene_export.argtypes = [P, P, C.POINTER(U32), C.POINTER(U32), P, P]
    L.gpugi_scene_set_hierarchy_ndf.argtypes = [P, P, P]
    L.gpugi_scene_set_triangle_test.argtypes = [P, P, U32]
    L.gpugi_scene_set_textures.argtypes = [P, P, P, U32, P]
    L.gpugi_hierarchy_importance.argtypes = [P, P, P, U32, U32, P, U32, U32]
    L.gpugi_hierarchy_read.argtypes = [P, P, P, P, P]
    for name in ("gpugi_trace_closest", "gpugi_trace_closest_device"):
        getattr(L, name).argtypes = [P, P] + [P] * 7 + [U64] + [P] * 4
    for name in ("gpugi_trace_any", "gpugi_trace_any_device"):
        getattr(L, name).argtypes = [P, P] + [P] * 7 + [U64, P]
    L.gpugi_trace_closest_device_async.argtypes = [P, P] + [P] * 7 + [U64] + [P] * 4 + [P]
    L.gpugi_trace_any_device_async.argtypes = [P, P] + [P] * 7 + [U64, P, P]
    L.gpugi_set_trace_config.argtypes = [P, U32, U32]
    L.gpugi_set_scene_layout.argtypes = [P, U32, U32]
    L.gpugi_set_host_pipeline.argtypes = [P, U32, U32]
    L.gpugi_trace_stats_device.argtypes = [P, P] + [P] * 7 + [U64, U32, P]
    for name, args in _EXTRA_DECLS.items():
        if hasattr(L, name):
            getattr(L, name).argtypes = args


# Signatures of the renderer entry points, filled in by render.py.
_EXTRA_DECLS: dict = {}


# Live handles, closed at interpreter exit in dependency order (caches,
# images and scenes before their contexts) while the library and the CUDA
# runtime are still loaded.
_LIVE: "weakref.WeakKeyDictionary" = weakref.WeakKeyDictionary()


def _register(obj, rank: int) -> None:
    _LIVE[obj] = rank


@atexit.register
def _close_all() -> None:
    for obj, _ in sorted(list(_LIVE.items()), key=lambda kv: kv[1]):
        try:
            obj.close()
        except Exception:
            pass


def _ptr(a):
    """Pointer of a numpy array or a torch tensor (host or device)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        assert a.flags["C_CONTIGUOUS"]
        return C.c_void_p(a.ctypes.data)
    return C.c_void_p(a.data_ptr())


class Context:
    def __init__(self, device: int = 0):
        self._h = C.c_void_p()

        class Opts(C.Structure):
            _fields_ = [("device", C.c_int), ("flags", C.c_uint32)]

        opts = Opts(device, 0)
        st = lib().gpugi_create(C.byref(self._h), C.byref(opts))
        if st != 0:
            raise GpugiError(st, "gpugi_create failed (no CUDA device?)")
        _register(self, 3)

    @property
    def handle(self):
        return self._h

    def check(self, st: int):
        if st != 0:
            raise GpugiError(st, lib().gpugi_last_error(self._h).decode())

    def sync(self):
        self.check(lib().gpugi_sync(self._h))

    def debug_raise_device_error(self, bits: int) -> None:
        """Test support: set device error bits as a device guard would."""
        self.check(lib().gpugi_debug_raise_device_error(self._h, bits))

    def device_error_bits(self) -> int:
        b = C.c_uint32()
        self.check(lib().gpugi_device_error_bits(self._h, C.byref(b)))
        return b.value

    @property
    def stream(self) -> int:
        return lib().gpugi_stream(self._h) or 0

    def set_trace_config(self, mode: int = 3, block_size: int = 128):
        self.check(lib().gpugi_set_trace_config(self._h, mode, block_size))

    def set_host_pipeline(self, parts: int = 2, zero_copy: bool = False):
        """Host-pointer queries: staging split into `parts` overlapping parts (1: no overlap),
        or kernels accessing page-locked arrays directly (zero_copy)."""
        self.check(lib().gpugi_set_host_pipeline(self._h, parts, int(bool(zero_copy))))

    def set_async_walker_share(self, percent: int = 50):
        """Percent of the persistent walker grid a stream-ordered device-array query launches."""
        self.check(lib().gpugi_set_async_walker_share(self._h, int(percent)))

    def set_scene_layout(self, shared_nodes: int = 0, render_shared_nodes: int = 0):
        """Top-of-tree nodes staged in shared memory, for scenes uploaded afterwards."""
        self.check(lib().gpugi_set_scene_layout(self._h, shared_nodes, render_shared_nodes))

    def autotune(self, scene: "DeviceScene", trace: bool = True, batch: bool = False) -> dict:
        """gpugi_autotune: times candidate launch settings on the scene and applies the fastest."""

        class Tuning(C.Structure):
            _fields_ = [("traceMode", C.c_uint32), ("traceBlock", C.c_uint32), ("batchPaths", C.c_uint32),
                        ("traceMraysPerSecond", C.c_double), ("batchMpathsPerSecond", C.c_double)]

        t = Tuning()
        L = lib()
        L.gpugi_autotune.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.POINTER(Tuning)]
        self.check(L.gpugi_autotune(self._h, scene.handle, (1 if trace else 0) | (2 if batch else 0), C.byref(t)))
        return {k: getattr(t, k) for k, _ in Tuning._fields_}

    def close(self):
        if self._h:
            lib().gpugi_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload_scene(self, bvh, positions, vertex_info=None, materials=None) -> "DeviceScene":
        return DeviceScene(self, bvh, positions, vertex_info, materials)

    def build_scene(self, positions, triangles, vertex_info=None, materials=None, leaf_size: int = 8) -> "DeviceScene":
        """Scene whose hierarchy is built on the GPU (gpugi_scene_build)."""
        return DeviceScene(self, None, positions, vertex_info, materials, triangles=triangles, leaf_size=leaf_size)


class DeviceScene:
    def __init__(self, ctx: Context, bvh, positions, vertex_info=None, materials=None, triangles=None,
                 leaf_size: int = 8):
        self.ctx = ctx
        self._h = C.c_void_p()
        if bvh is None:
            tris = np.ascontiguousarray(triangles, dtype=np.uint32)
            pos = np.ascontiguousarray(positions, dtype=np.float32)
            vi = None if vertex_info is None else np.ascontiguousarray(vertex_info, dtype=np.float32)
            mats = None if materials is None else np.ascontiguousarray(materials, dtype=np.float32).reshape(-1, 24)
            nm = 0 if mats is None else mats.shape[0]
            ctx.check(lib().gpugi_scene_build(ctx.handle, _ptr(pos), pos.shape[0], _ptr(tris), tris.shape[0],
                                              _ptr(vi), _ptr(mats), nm, leaf_size, C.byref(self._h)))
            _register(self, 2)
            nn, ns = C.c_uint32(), C.c_uint32()
            ctx.check(lib().gpugi_scene_export(ctx.handle, self._h, C.byref(nn), C.byref(ns), None, None))
            self.num_nodes, self.num_slots, self.leaf_size = nn.value, ns.value, leaf_size
            self.bounds_kind = 0
            return
        hier = np.ascontiguousarray(bvh.hierarchy, dtype=np.float32)
        slots = np.ascontiguousarray(bvh.slots, dtype=np.int32)
        pos = np.ascontiguousarray(positions, dtype=np.float32)
        vi = None if vertex_info is None else np.ascontiguousarray(vertex_info, dtype=np.float32)
        mats = None if materials is None else np.ascontiguousarray(materials, dtype=np.float32).reshape(-1, 24)
        nm = 0 if mats is None else mats.shape[0]
        st = lib().gpugi_scene_upload(ctx.handle, _ptr(hier), hier.shape[0], bvh.bounds_kind, _ptr(slots),
                                      slots.shape[0], bvh.leaf_size, _ptr(pos), _ptr(vi), pos.shape[0], _ptr(mats),
                                      nm, C.byref(self._h))
        ctx.check(st)
        _register(self, 2)
        self.num_nodes = hier.shape[0]
        self.num_slots = slots.shape[0]
        self.leaf_size = bvh.leaf_size
        self.bounds_kind = bvh.bounds_kind

    def export(self):
        """The scene's hierarchy and leaf slots as a bvh.BVH (device node order)."""
        from . import bvh as B
        nn, ns = C.c_uint32(), C.c_uint32()
        self.ctx.check(lib().gpugi_scene_export(self.ctx.handle, self._h, C.byref(nn), C.byref(ns), None, None))
        hier = np.zeros((nn.value, 12 if self.bounds_kind == 2 else 8), np.float32)
        slots = np.zeros((ns.value, 4), np.int32)
        self.ctx.check(lib().gpugi_scene_export(self.ctx.handle, self._h, C.byref(nn), C.byref(ns), _ptr(hier),
                                                _ptr(slots)))
        child = hier[:, 3].view(np.uint32)
        parents = np.zeros(nn.value, np.uint32)
        inner = np.nonzero((child & 0x80000000) == 0)[0]
        left = child[inner]
        parents[left] = inner
        parents[hier[left, 7].view(np.uint32)] = inner
        return B.BVH(hierarchy=hier, slots=slots, parents=parents, leaf_size=self.leaf_size, bounds_kind=self.bounds_kind,
                     max_depth=0)

    def set_triangle_test(self, watertight: bool) -> None:
        """Triangle test of the ray queries on this scene: the reference's
        (False) or the watertight test (True), gpugi_scene_set_triangle_test."""
        self.ctx.check(lib().gpugi_scene_set_triangle_test(self.ctx.handle, self._h, 1 if watertight else 0))

    def set_textures(self, textures, material_textures) -> None:
        """Material textures (gpugi_scene_set_textures): textures is a list
        of float32 (height, width, 4) RGBA arrays (row 0 at t = 0),
        material_textures int32 (numMaterials, 4): the texture of each
        material's {reflectiveness, opacity, diffuse, emissivity} map or -1.
        An empty list removes the textures."""

        class Tex(C.Structure):
            _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("rgba", C.c_void_p)]

        keep = [np.ascontiguousarray(t, dtype=np.float32) for t in textures]
        arr = (Tex * max(1, len(keep)))()
        for i, t in enumerate(keep):
            assert t.ndim == 3 and t.shape[2] == 4
            arr[i] = Tex(t.shape[1], t.shape[0], t.ctypes.data)
        mt = np.ascontiguousarray(material_textures if keep else np.zeros((0, 4)), dtype=np.int32)
        self.ctx.check(lib().gpugi_scene_set_textures(self.ctx.handle, self._h, C.cast(arr, C.c_void_p), len(keep),
                                                      _ptr(mt) if keep else None))

    def set_hierarchy_ndf(self, sggx: np.ndarray) -> None:
        """Node NDFs (uint16 [numNodes, 6], bvhmake's approx_sggx in the
        uploaded node order) and the node materials of the hierarchy-
        importance renderer."""
        a = np.ascontiguousarray(sggx, dtype=np.uint16)
        if a.shape != (self.num_nodes, 6):
            raise ValueError("sggx must be uint16 [numNodes, 6]")
        self.ctx.check(lib().gpugi_scene_set_hierarchy_ndf(self.ctx.handle, self._h, _ptr(a)))

    def hierarchy_importance(self, camera, width: int, height: int, light_samples: np.ndarray,
                             iterations: int = 10) -> None:
        """The importance pass (acquisition + propagation) with one light-sample set."""
        ls = np.ascontiguousarray(light_samples, dtype=np.float32).reshape(-1, 8)
        self.ctx.check(lib().gpugi_hierarchy_importance(self.ctx.handle, self._h, C.byref(camera), width, height,
                                                        _ptr(ls), ls.shape[0], iterations))

    def hierarchy_read(self):
        """(importance float32 [numNodes + numSlots, 2], subtree float32
        [numNodes], node materials uint32 [numNodes, 12]) in the uploaded order."""
        imp = np.zeros((self.num_nodes + self.num_slots, 2), np.float32)
        sub = np.zeros(self.num_nodes, np.float32)
        mats = np.zeros((self.num_nodes, 12), np.uint32)
        self.ctx.check(lib().gpugi_hierarchy_read(self.ctx.handle, self._h, _ptr(imp), _ptr(sub), _ptr(mats)))
        return imp, sub, mats

    @property
    def handle(self):
        return self._h

    def close(self):
        if self._h:
            lib().gpugi_scene_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


RAY_KEYS = ("ox", "oy", "oz", "dx", "dy", "dz", "tmax")


def trace_closest(ctx: Context, scene: DeviceScene, rays: dict) -> dict:
    """Host arrays in, host arrays out (copies through the context)."""
    r = [np.ascontiguousarray(rays[k], dtype=np.float32) for k in RAY_KEYS]
    n = r[0].shape[0]
    out = dict(slot=np.empty(n, np.int32), t=np.empty(n, np.float32), u=np.empty(n, np.float32),
               v=np.empty(n, np.float32))
    ctx.check(lib().gpugi_trace_closest(ctx.handle, scene.handle, *[_ptr(a) for a in r], n, _ptr(out["slot"]),
                                        _ptr(out["t"]), _ptr(out["u"]), _ptr(out["v"])))
    return out


def trace_any(ctx: Context, scene: DeviceScene, rays: dict) -> np.ndarray:
    r = [np.ascontiguousarray(rays[k], dtype=np.float32) for k in RAY_KEYS]
    n = r[0].shape[0]
    occ = np.empty(n, np.uint8)
    ctx.check(lib().gpugi_trace_any(ctx.handle, scene.handle, *[_ptr(a) for a in r], n, _ptr(occ)))
    return occ


def trace_closest_device(ctx: Context, scene: DeviceScene, rays: dict, out: dict) -> None:
    """Device tensors (torch) in and out; asynchronous on the context stream."""
    n = rays["ox"].numel()
    ctx.check(lib().gpugi_trace_closest_device(ctx.handle, scene.handle, *[_ptr(rays[k]) for k in RAY_KEYS], n,
                                               _ptr(out["slot"]), _ptr(out["t"]), _ptr(out["u"]), _ptr(out["v"])))


def trace_closest_device_async(ctx: Context, scene: DeviceScene, rays: dict, out: dict, stream: int) -> None:
    """As trace_closest_device, enqueued on a caller stream (a cudaStream_t
    handle, e.g. torch's Stream.cuda_stream; 0 = the context stream)."""
    n = rays["ox"].numel()
    ctx.check(lib().gpugi_trace_closest_device_async(ctx.handle, scene.handle, *[_ptr(rays[k]) for k in RAY_KEYS], n,
                                                     _ptr(out["slot"]), _ptr(out["t"]), _ptr(out["u"]), _ptr(out["v"]),
                                                     C.c_void_p(stream or None)))


def trace_any_device_async(ctx: Context, scene: DeviceScene, rays: dict, occluded, stream: int) -> None:
    n = rays["ox"].numel()
    ctx.check(lib().gpugi_trace_any_device_async(ctx.handle, scene.handle, *[_ptr(rays[k]) for k in RAY_KEYS], n,
                                                 _ptr(occluded), C.c_void_p(stream or None)))


def trace_any_device(ctx: Context, scene: DeviceScene, rays: dict, occluded) -> None:
    n = rays["ox"].numel()
    ctx.check(lib().gpugi_trace_any_device(ctx.handle, scene.handle, *[_ptr(rays[k]) for k in RAY_KEYS], n,
                                           _ptr(occluded)))


def trace_stats_device(ctx: Context, scene: DeviceScene, rays: dict, any_hit: bool = False) -> np.ndarray:
    """Sums over the rays of (nodes visited, leaf slots fetched, valid triangles tested)."""
    n = rays["ox"].numel()
    sums = np.zeros(3, np.uint64)
    ctx.check(lib().gpugi_trace_stats_device(ctx.handle, scene.handle, *[_ptr(rays[k]) for k in RAY_KEYS], n,
                                             int(any_hit), _ptr(sums)))
    return sums


def algorithmic_bytes(sums: np.ndarray, n_rays: int, any_hit: bool = False) -> int:
    """gpugi's own fetch pattern per ray: 24 B ray in + 16 B out (4 B any-hit)
    + 32 B per node + 16 B per leaf slot + 36 B per valid triangle
    (gpugi/scene/scene.hpp:30-38, traceray.glsl:126,137-139)."""
    s = [int(x) for x in sums]
    return n_rays * (24 + (4 if any_hit else 16)) + 32 * s[0] + 16 * s[1] + 36 * s[2]


def vertex_info(normals: np.ndarray, texcoords: np.ndarray) -> np.ndarray:
    """VertexInfo {atan2(n.y, n.x), n.z, u, v} per vertex (gpugi/scene/scene.cpp:79-84)."""
    n = np.asarray(normals, dtype=np.float32)
    out = np.zeros((n.shape[0], 4), dtype=np.float32)
    out[:, 0] = np.arctan2(n[:, 1], n[:, 0])
    out[:, 1] = n[:, 2]
    out[:, 2:4] = texcoords
    return out
