"""Python front end of the neural radiance cache entry points (gpugi_nrc_*)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import cuda

PARAMS = 17408
KERNELS = {"tcgen05": 0, "mma_sync": 1}
LAYER_SHAPES = [(64, 64)] * 4 + [(64, 16)]  # (in, out) per layer, output padded to 16


def _declare():
    L = cuda.lib()
    if getattr(L, "_nrc_declared", False):
        return L
    P, U64, F = C.c_void_p, C.c_uint64, C.c_float
    L.gpugi_nrc_create.argtypes = [P, P, P, U64, F, C.POINTER(P)]
    L.gpugi_nrc_destroy.argtypes = [P]
    L.gpugi_nrc_destroy.restype = None
    L.gpugi_nrc_get_weights.argtypes = [P, P, P]
    L.gpugi_nrc_set_weights.argtypes = [P, P, P]
    L.gpugi_nrc_infer_device.argtypes = [P, P, P, U64, P]
    L.gpugi_nrc_train_device.argtypes = [P, P, P, U64, P]
    L.gpugi_nrc_gradient_device.argtypes = [P, P, P, U64, P, P, P]
    L.gpugi_nrc_encode_device.argtypes = [P, P, P, U64, P]
    L.gpugi_nrc_set_ema.argtypes = [P, P, F]
    L.gpugi_nrc_set_kernels.argtypes = [P, P, C.c_uint32]
    from . import render
    render._declare()
    L.gpugi_render_nrc.argtypes = [P, P, C.POINTER(render.Camera), C.POINTER(render.RenderParams), P,
                                   C.POINTER(C.c_uint64), P, C.POINTER(NrcParams), P]
    L._nrc_declared = True
    return L


class NrcParams(C.Structure):
    _fields_ = [("terminateDepth", C.c_uint32), ("trainFraction", C.c_float), ("maxTrainSamples", C.c_uint32),
                ("trainSteps", C.c_uint32), ("train", C.c_uint32), ("samplesPerFrame", C.c_uint32),
                ("trainLength", C.c_uint32), ("unbiasedFraction", C.c_float), ("terminateSpread", C.c_float),
                ("lanes", C.c_uint32)]


def _torch_to_ctx():
    """The library works on its own stream: finish torch's pending work on
    the tensors first (results are made visible by ctx.sync afterwards)."""
    import torch
    torch.cuda.current_stream().synchronize()


def unflatten(w: np.ndarray) -> list[np.ndarray]:
    """Flat master weights -> per-layer [in, out] matrices."""
    out, off = [], 0
    for i, o in LAYER_SHAPES:
        out.append(w[off:off + i * o].reshape(i, o))
        off += 64 * 64
    return out


class RadianceCache:
    def __init__(self, ctx: cuda.Context, box_min, box_max, seed: int = 1, learning_rate: float = 1e-2):
        self.ctx = ctx
        self._h = C.c_void_p()
        L = _declare()
        bmin = (C.c_float * 3)(*map(float, box_min))
        bmax = (C.c_float * 3)(*map(float, box_max))
        ctx.check(L.gpugi_nrc_create(ctx.handle, bmin, bmax, seed, float(learning_rate), C.byref(self._h)))
        cuda._register(self, 0)

    @property
    def handle(self):
        return self._h

    def weights(self) -> np.ndarray:
        w = np.zeros(PARAMS, np.float32)
        self.ctx.check(_declare().gpugi_nrc_get_weights(self.ctx.handle, self._h, cuda._ptr(w)))
        return w

    def set_weights(self, w: np.ndarray):
        w = np.ascontiguousarray(w, np.float32)
        assert w.shape == (PARAMS,)
        self.ctx.check(_declare().gpugi_nrc_set_weights(self.ctx.handle, self._h, cuda._ptr(w)))

    def set_kernels(self, kernels: str):
        """Training kernels: "tcgen05" (default) or "mma_sync"."""
        self.ctx.check(_declare().gpugi_nrc_set_kernels(self.ctx.handle, self._h, KERNELS[kernels]))

    def set_ema(self, decay: float):
        """Decay of the moving average of the weights that inference uses (0: the trained weights)."""
        self.ctx.check(_declare().gpugi_nrc_set_ema(self.ctx.handle, self._h, float(decay)))

    def infer(self, queries) -> "object":
        """queries: torch (n, 12) float32 cuda tensor -> (n, 3) radiance tensor."""
        import torch
        n = queries.shape[0]
        out = torch.empty((n, 3), dtype=torch.float32, device=queries.device)
        _torch_to_ctx()
        self.ctx.check(_declare().gpugi_nrc_infer_device(self.ctx.handle, self._h, cuda._ptr(queries), n,
                                                         cuda._ptr(out)))
        self.ctx.sync()
        return out

    def train(self, samples, want_loss: bool = True) -> float | None:
        """One Adam step on a torch (n, 15) float32 cuda tensor."""
        loss = C.c_float()
        _torch_to_ctx()
        self.ctx.check(_declare().gpugi_nrc_train_device(self.ctx.handle, self._h, cuda._ptr(samples),
                                                         samples.shape[0], C.byref(loss) if want_loss else None))
        self.ctx.sync()  # the samples tensor may be released by the caller right after
        return loss.value if want_loss else None

    def gradient(self, samples):
        n = samples.shape[0]
        pred = np.zeros((n, 3), np.float32)
        grad = np.zeros(PARAMS, np.float32)
        loss = C.c_float()
        _torch_to_ctx()
        self.ctx.check(_declare().gpugi_nrc_gradient_device(self.ctx.handle, self._h, cuda._ptr(samples), n,
                                                            cuda._ptr(pred), cuda._ptr(grad), C.byref(loss)))
        return pred, grad, loss.value

    def encode(self, queries):
        import torch
        n = queries.shape[0]
        out = torch.empty((n, 64), dtype=torch.float16, device=queries.device)
        _torch_to_ctx()
        self.ctx.check(_declare().gpugi_nrc_encode_device(self.ctx.handle, self._h, cuda._ptr(queries), n,
                                                          cuda._ptr(out)))
        self.ctx.sync()
        return out

    def close(self):
        if self._h:
            _declare().gpugi_nrc_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def render_nrc(ctx: cuda.Context, scene: cuda.DeviceScene, camera, image, cache: RadianceCache,
               max_path_length: int = 8, samples: int = 1, iteration: int = 0, num_light_samples: int = 128,
               sky=(0.0, 0.0, 0.0), rr_start_depth: int = 0, light_samples: np.ndarray | None = None,
               rng_state: list | None = None, terminate_depth: int = 1, train_fraction: float = 0.03,
               max_train_samples: int = 65536, train_steps: int = 1, train: bool = True,
               samples_per_frame: int = 1, pass_: str = "PT", rng: str = "pcg", train_length: int = 0,
               unbiased_fraction: float = 1.0 / 16.0, terminate_spread: float = 0.0, lanes: int = 4) -> None:
    """`samples` iterations of path tracing (pass_ "PT") or bidirectional
    path tracing ("BPT") with the radiance cache (gpugi_render_nrc); rng
    selects the random streams as in render.render. train_length >= 1
    turns on self-training (training paths stop at that vertex and take the
    cache's radiance, except unbiased_fraction of them); terminate_spread > 0
    stops PT render paths by path spread (0.01 in the NRC paper), at vertex
    terminate_depth at the latest. lanes: frames in flight (1-4)."""
    from . import render
    L = _declare()
    if pass_ not in ("PT", "BPT"):
        raise ValueError("the radiance cache serves the PT and BPT passes")
    p = render.RenderParams(render.PASSES[pass_], image.width, image.height, max_path_length, rr_start_depth,
                            iteration, samples, num_light_samples, render._f3(sky), render.RNG_FLAGS[rng])
    ls = None if light_samples is None else np.ascontiguousarray(light_samples, dtype=np.float32)
    if ls is not None:
        assert ls.shape == (samples, num_light_samples, 8)
    q = NrcParams(terminate_depth, float(train_fraction), max_train_samples, train_steps, int(bool(train)),
                  samples_per_frame, train_length, float(unbiased_fraction), float(terminate_spread), lanes)
    st = C.c_uint64(rng_state[0] if rng_state else 0)
    ctx.check(L.gpugi_render_nrc(ctx.handle, scene.handle, C.byref(camera), C.byref(p), cuda._ptr(ls),
                                 C.byref(st) if ls is None else None, cache.handle, C.byref(q), image.handle))
    if rng_state is not None and ls is None:
        rng_state[0] = st.value


def smoke_check(ctx: cuda.Context) -> None:
    """The cache's tcgen05 kernels on a small batch (used by smoke()): the
    training step's loss and gradient agree with the mma.sync kernels, and
    inference is finite."""
    import torch
    rng = np.random.default_rng(1)
    n = 2000
    q = np.concatenate([rng.uniform(-1, 1, (n, 3)), rng.normal(size=(n, 3)), rng.normal(size=(n, 3)),
                        rng.uniform(0.1, 0.9, (n, 3))], 1).astype(np.float32)
    q[:, 3:6] /= np.linalg.norm(q[:, 3:6], axis=1, keepdims=True)
    q[:, 6:9] /= np.linalg.norm(q[:, 6:9], axis=1, keepdims=True)
    samples = torch.from_numpy(np.concatenate([q, rng.uniform(0, 1, (n, 3)).astype(np.float32)], 1)).cuda()
    c = RadianceCache(ctx, (-1, -1, -1), (1, 1, 1), seed=3)
    try:
        out = {}
        for k in ("mma_sync", "tcgen05"):
            c.set_kernels(k)
            out[k] = c.gradient(samples)
        (_, g0, l0), (_, g1, l1) = out["mma_sync"], out["tcgen05"]
        assert abs(l1 / l0 - 1) < 1e-2, (l0, l1)
        assert np.linalg.norm(g1 - g0) <= 2e-2 * np.linalg.norm(g0), "tcgen05 gradient differs"
        c.train(samples)
        r = c.infer(samples[:, :12].contiguous()).cpu().numpy()
        assert np.isfinite(r).all() and ctx.device_error_bits() == 0
    finally:
        c.close()

