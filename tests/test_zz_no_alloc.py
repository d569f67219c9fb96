"""gpugi_trace_closest_noalloc: closest-hit queries for callers that cannot
let the library allocate device memory (an engine that owns all device
memory through its own pool, or a frame loop where cudaMalloc would
synchronise the device). Its scratch is a static device array in the
library, so the call allocates nothing.

Checked through the C ABI against the allocating entry point
(gpugi_trace_closest_device) on the same device inputs: the results must be
bit-identical, the same bar as every traversal test, on two calls in a row
(the static scratch keeps the previous call's contents and must be reset by
the call itself). The file is named to run last so that a `-x` run has
finished every other test before it; it also passes alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from gpugi_gb300 import bvh, cuda, scenes

pytestmark = pytest.mark.gpu

MAX_RAYS = 1 << 20  # GPUGI_NOALLOC_MAX_RAYS


def _bind():
    L = cuda.lib()
    P, U64 = C.c_void_p, C.c_uint64
    L.gpugi_trace_closest_noalloc.argtypes = [P, P] + [P] * 7 + [U64] + [P] * 4
    return L


def _outputs(torch, n):
    return dict(slot=torch.full((n,), -7, dtype=torch.int32, device="cuda"),
                t=torch.full((n,), -1.0, device="cuda"), u=torch.full((n,), -1.0, device="cuda"),
                v=torch.full((n,), -1.0, device="cuda"))


def _noalloc(L, ctx, ds, rays, out, n):
    return L.gpugi_trace_closest_noalloc(ctx.handle, ds.handle, *[cuda._ptr(rays[k]) for k in cuda.RAY_KEYS], n,
                                         cuda._ptr(out["slot"]), cuda._ptr(out["t"]), cuda._ptr(out["u"]),
                                         cuda._ptr(out["v"]))


def test_noalloc_matches_allocating_entry_point(built):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    L = _bind()
    ctx = cuda.Context(0)
    sc = scenes.displaced_icosphere(65536, seed=1)
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep")
    ds = ctx.upload_scene(b, sc["positions"])
    batches = [scenes.random_rays(MAX_RAYS, seed=41),                       # the full limit, mostly misses
               scenes.aimed_rays(200_003, sc["positions"], seed=42)]       # a ragged size, mostly hits
    for rays_np in batches:
        n = rays_np["ox"].shape[0]
        rays = {k: torch.from_numpy(rays_np[k]).cuda() for k in cuda.RAY_KEYS}
        ref = _outputs(torch, n)
        cuda.trace_closest_device(ctx, ds, rays, ref)
        ctx.sync()
        expect = {k: v.cpu().numpy() for k, v in ref.items()}
        for call in range(2):  # two calls in a row share the static scratch
            out = _outputs(torch, n)
            ctx.check(_noalloc(L, ctx, ds, rays, out, n))
            ctx.sync()
            got = {k: v.cpu().numpy() for k, v in out.items()}
            assert np.array_equal(got["slot"], expect["slot"]), f"call {call}: slot mismatch"
            for k in ("t", "u", "v"):
                assert np.array_equal(got[k].view(np.uint32), expect[k].view(np.uint32)), f"call {call}: {k}"
    # beyond the stated maximum the call is refused before touching the GPU
    too_many = MAX_RAYS + 1
    rays = {k: torch.zeros(too_many, device="cuda") for k in cuda.RAY_KEYS}
    out = _outputs(torch, too_many)
    st = _noalloc(L, ctx, ds, rays, out, too_many)
    assert st == 1  # GPUGI_ERROR_INVALID_ARGUMENT
    assert b"GPUGI_NOALLOC_MAX_RAYS" in cuda.lib().gpugi_last_error(ctx.handle)
    assert ctx.device_error_bits() == 0
    ds.close()
    ctx.close()
