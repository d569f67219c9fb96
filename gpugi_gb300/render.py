"""Python front end of the rendering entry points of libgpugi_cuda.so.

Thin ctypes bindings of gpugi_render / gpugi_image_* / gpugi_camera_lookat /
gpugi_generate_light_samples (include/gpugi_cuda.h). No compute here.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import cuda

PASSES = {"PT": 0, "LT": 1, "BPT": 2, "WHITTED": 3, "PM": 4, "HIERARCHY": 5, "IM": 6}
# Initial light samples per iteration as each renderer configures them
# (pathtracer.cpp:28, lightpathtracer.cpp:16, bidirectionalpathtracer.cpp:160).
DEFAULT_LIGHT_SAMPLES = {"PT": 128, "LT": 256, "BPT": 128, "WHITTED": 128, "PM": 128, "HIERARCHY": 128, "IM": 128}
# Random streams (gpugi_render_params.flags): "pcg" (the default) or
# "reference" (GPUGI_RENDER_REFERENCE_RNG: gpugi's wanghash + xorshift32).
RNG_FLAGS = {"pcg": 0, "reference": 1}


class Camera(C.Structure):
    _fields_ = [("U", C.c_float * 3), ("V", C.c_float * 3), ("W", C.c_float * 3), ("position", C.c_float * 3),
                ("pixelArea", C.c_float)]

    def as_array(self) -> np.ndarray:
        return np.array(list(self.U) + list(self.V) + list(self.W) + list(self.position) + [self.pixelArea],
                        dtype=np.float32)


class RenderParams(C.Structure):
    _fields_ = [("pass_", C.c_uint32), ("width", C.c_uint32), ("height", C.c_uint32),
                ("maxPathLength", C.c_uint32), ("rrStartDepth", C.c_uint32), ("iteration", C.c_uint32),
                ("samples", C.c_uint32), ("numLightSamples", C.c_uint32), ("sky", C.c_float * 3),
                ("flags", C.c_uint32)]


def _declare():
    L = cuda.lib()
    if getattr(L, "_render_declared", False):
        return L
    P, U32, U64, D = C.c_void_p, C.c_uint32, C.c_uint64, C.c_double
    L.gpugi_camera_lookat.argtypes = [P, P, P, C.c_float, U32, U32, C.POINTER(Camera)]
    L.gpugi_image_create.argtypes = [P, U32, U32, U32, C.POINTER(P)]
    L.gpugi_image_destroy.argtypes = [P]
    L.gpugi_image_destroy.restype = None
    L.gpugi_image_clear.argtypes = [P, P]
    L.gpugi_image_read.argtypes = [P, P, P, P]
    L.gpugi_image_write.argtypes = [P, P, P, P]
    L.gpugi_image_mse.argtypes = [P, P, D, P, U32, C.POINTER(D)]
    L.gpugi_scene_add_point_light.argtypes = [P, P, P]
    L.gpugi_scene_add_directional_light.argtypes = [P, P, P]
    L.gpugi_generate_light_samples.argtypes = [P, C.POINTER(U64), U32, P]
    L.gpugi_render.argtypes = [P, P, C.POINTER(Camera), C.POINTER(RenderParams), P, C.POINTER(U64), P]
    L.gpugi_render_ray_counts.argtypes = [P, P]
    L.gpugi_render_batch.argtypes = [P, P, U32]
    L.gpugi_set_batch_config.argtypes = [P, U32, U32]
    L.gpugi_set_photon_config.argtypes = [P, U32, C.c_float, U32]
    L.gpugi_set_importon_config.argtypes = [P, U32, C.c_float, U32]
    L._render_declared = True
    return L


def _f3(v):
    return (C.c_float * 3)(*[float(x) for x in v])


def camera_lookat(position, lookat, up, yfov_deg: float, width: int, height: int) -> Camera:
    cam = Camera()
    st = _declare().gpugi_camera_lookat(_f3(position), _f3(lookat), _f3(up), float(yfov_deg), width, height,
                                        C.byref(cam))
    if st != 0:
        raise cuda.GpugiError(st, "gpugi_camera_lookat failed")
    return cam


class Image:
    def __init__(self, ctx: cuda.Context, width: int, height: int, fp64: bool = False):
        self.ctx, self.width, self.height = ctx, width, height
        self.fp64 = fp64
        self._h = C.c_void_p()
        ctx.check(_declare().gpugi_image_create(ctx.handle, width, height, 1 if fp64 else 0, C.byref(self._h)))
        cuda._register(self, 1)

    @property
    def handle(self):
        return self._h

    def clear(self):
        self.ctx.check(_declare().gpugi_image_clear(self.ctx.handle, self._h))

    def read(self) -> np.ndarray:
        out = np.zeros((self.height, self.width, 4), np.float32)
        self.ctx.check(_declare().gpugi_image_read(self.ctx.handle, self._h, cuda._ptr(out), None))
        return out

    def read64(self) -> np.ndarray:
        out = np.zeros((self.height, self.width, 3), np.float64)
        self.ctx.check(_declare().gpugi_image_read(self.ctx.handle, self._h, None, cuda._ptr(out)))
        return out

    def write(self, rgba: np.ndarray, rgb64: np.ndarray | None = None) -> None:
        """Replace the sums (gpugi_image_write); rgb64 None zeroes an FP64 accumulation."""
        a = np.ascontiguousarray(rgba, dtype=np.float32)
        assert a.shape == (self.height, self.width, 4)
        b = None if rgb64 is None else np.ascontiguousarray(rgb64, dtype=np.float64)
        assert b is None or b.shape == (self.height, self.width, 3)
        self.ctx.check(_declare().gpugi_image_write(self.ctx.handle, self._h, cuda._ptr(a),
                                                    None if b is None else cuda._ptr(b)))

    def mse(self, divisor: float, reference: np.ndarray, use_fp64: bool = False) -> float:
        ref = np.ascontiguousarray(reference[..., :3], dtype=np.float32)
        out = C.c_double()
        self.ctx.check(_declare().gpugi_image_mse(self.ctx.handle, self._h, float(divisor), cuda._ptr(ref),
                                                  1 if use_fp64 else 0, C.byref(out)))
        return out.value

    def close(self):
        if self._h:
            _declare().gpugi_image_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def add_point_light(scene: cuda.DeviceScene, position, intensity):
    scene.ctx.check(_declare().gpugi_scene_add_point_light(scene.handle, _f3(position), _f3(intensity)))


def add_directional_light(scene: cuda.DeviceScene, towards_light, irradiance):
    scene.ctx.check(_declare().gpugi_scene_add_directional_light(scene.handle, _f3(towards_light),
                                                                 _f3(irradiance)))


def generate_light_samples(scene: cuda.DeviceScene, rng_state: list, n: int) -> np.ndarray:
    """Host LightSampler; rng_state is a one-element list holding the xorshift64 state."""
    out = np.zeros((n, 8), np.float32)
    st = C.c_uint64(rng_state[0])
    scene.ctx.check(_declare().gpugi_generate_light_samples(scene.handle, C.byref(st), n, cuda._ptr(out)))
    rng_state[0] = st.value
    return out


def render(ctx: cuda.Context, scene: cuda.DeviceScene, camera: Camera, image: Image, pass_: str = "PT",
           max_path_length: int = 8, samples: int = 1, iteration: int = 0, num_light_samples: int | None = None,
           sky=(0.0, 0.0, 0.0), rr_start_depth: int = 0, light_samples: np.ndarray | None = None,
           rng_state: list | None = None, rng: str = "pcg") -> None:
    """Render `samples` iterations of a pass into the image (asynchronous).

    light_samples: (samples, numLightSamples, 8) float32, or None to let the
    library's host sampler draw them from rng_state (a one-element list).
    rng: the paths' random streams, "pcg" or "reference"."""
    L = _declare()
    nls = num_light_samples or DEFAULT_LIGHT_SAMPLES[pass_]
    p = RenderParams(PASSES[pass_], image.width, image.height, max_path_length, rr_start_depth, iteration, samples,
                     nls, _f3(sky), RNG_FLAGS[rng])
    ls = None if light_samples is None else np.ascontiguousarray(light_samples, dtype=np.float32)
    if ls is not None:
        assert ls.shape == (samples, nls, 8)
    st = C.c_uint64(rng_state[0] if rng_state else 0)
    ctx.check(L.gpugi_render(ctx.handle, scene.handle, C.byref(camera), C.byref(p), cuda._ptr(ls),
                             C.byref(st) if ls is None else None, image.handle))
    if rng_state is not None and ls is None:
        rng_state[0] = st.value


class Job(C.Structure):
    _fields_ = [("scene", C.c_void_p), ("camera", Camera), ("params", RenderParams), ("lightSamples", C.c_void_p),
                ("rngState", C.POINTER(C.c_uint64)), ("image", C.c_void_p)]


def render_batch(ctx: cuda.Context, jobs: list[dict]) -> None:
    """gpugi_render_batch over jobs given as dicts with the keys of render():
    scene, camera, image, pass_ (default PT), max_path_length, samples,
    iteration, num_light_samples, sky, rr_start_depth, rng, light_samples or
    rng_state (a one-element list, updated)."""
    L = _declare()
    arr = (Job * len(jobs))()
    keep, states = [], []
    for i, j in enumerate(jobs):
        pass_ = j.get("pass_", "PT")
        img = j["image"]
        nls = j.get("num_light_samples") or DEFAULT_LIGHT_SAMPLES[pass_]
        samples = j.get("samples", 1)
        p = RenderParams(PASSES[pass_], img.width, img.height, j.get("max_path_length", 8),
                         j.get("rr_start_depth", 0), j.get("iteration", 0), samples, nls,
                         _f3(j.get("sky", (0.0, 0.0, 0.0))), RNG_FLAGS[j.get("rng", "pcg")])
        ls = j.get("light_samples")
        st = None
        if ls is not None:
            ls = np.ascontiguousarray(ls, dtype=np.float32)
            assert ls.shape == (samples, nls, 8)
            keep.append(ls)
        else:
            st = C.c_uint64(j["rng_state"][0])
            states.append((st, j["rng_state"]))
        arr[i] = Job(j["scene"].handle, j["camera"], p, cuda._ptr(ls) if ls is not None else None,
                     C.pointer(st) if st is not None else None, img.handle)
    ctx.check(L.gpugi_render_batch(ctx.handle, arr, len(jobs)))
    for st, ref in states:
        ref[0] = st.value


def set_photon_config(ctx: cuda.Context, photons_per_light_sample: int = 2048, query_radius: float = 0.01,
                      progressive: bool = False) -> None:
    """Photon mapper settings (gpugi_set_photon_config)."""
    ctx.check(_declare().gpugi_set_photon_config(ctx.handle, photons_per_light_sample, float(query_radius),
                                                  int(bool(progressive))))


def set_importon_config(ctx: cuda.Context, photons_per_light_sample: int = 2048, query_radius: float = 0.005,
                      progressive: bool = False) -> None:
    """Importon map light tracer settings (gpugi_set_importon_config)."""
    ctx.check(_declare().gpugi_set_importon_config(ctx.handle, photons_per_light_sample, float(query_radius),
                                                  int(bool(progressive))))


def set_batch_config(ctx: cuda.Context, paths_per_round: int = 16 << 20, use_graph: bool = True) -> None:
    ctx.check(_declare().gpugi_set_batch_config(ctx.handle, paths_per_round, int(bool(use_graph))))


def ray_counts(ctx: cuda.Context) -> tuple[int, int]:
    c = np.zeros(2, np.uint64)
    ctx.check(_declare().gpugi_render_ray_counts(ctx.handle, cuda._ptr(c)))
    return int(c[0]), int(c[1])


def wanghash(x: int) -> int:
    """gpugi's WangHash (gpugi/utilities/random.cpp:5-13): FrameSeed of an iteration."""
    x &= 0xFFFFFFFF
    x = ((x ^ 61) ^ (x >> 16)) & 0xFFFFFFFF
    x = (x * 9) & 0xFFFFFFFF
    x ^= x >> 4
    x = (x * 0x27D4EB2D) & 0xFFFFFFFF
    x ^= x >> 15
    return x


def pcg_hash(x: int) -> int:
    """One PCG-RXS-M-XS-32 step used as a hash (the PCG streams' seeding)."""
    state = ((x & 0xFFFFFFFF) * 747796405 + 2891336453) & 0xFFFFFFFF
    w = (((state >> ((state >> 28) + 4)) ^ state) * 277803737) & 0xFFFFFFFF
    return ((w >> 22) ^ w) & 0xFFFFFFFF


def frame_seed(iteration: int, rng: str = "pcg") -> int:
    """FrameSeed of an iteration for the given random streams: WangHash
    (RendererSystem::PerIterationBufferUpdate, gpugi/renderer/renderersystem.cpp:101)
    or the PCG hash."""
    return pcg_hash(iteration) if rng == "pcg" else wanghash(iteration)


def smoke_check(ctx: cuda.Context) -> None:
    """One tiny PT iteration on the GPU, compared with the oracle (used by smoke())."""
    import oracle

    from . import bvh, scenes
    sc = scenes.cornell_room(seed=1, sphere_level=2, wall_grid=2)
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep")
    vi = cuda.vertex_info(sc["normals"], sc["texcoords"])
    ds = ctx.upload_scene(b, sc["positions"], vi, sc["materials"])
    w = h = 32
    cam = camera_lookat(*scenes.CORNELL_CAMERA, w, h)
    ls = generate_light_samples(ds, [123], 128)[None]
    img = Image(ctx, w, h)
    render(ctx, ds, cam, img, "PT", max_path_length=1, samples=1, iteration=0, light_samples=ls)
    g = img.read()[..., :3]
    o = oracle.render(b, sc, "PT", w, h, cam.as_array(), frame_seed(0), ls[0], max_path_length=1)[..., :3]
    err = np.abs(g - o).max() / max(1e-6, float(np.abs(o).max()))
    assert err < 1e-3, f"direct-light image differs from the oracle (max rel err {err})"
    img.close()
    ds.close()
