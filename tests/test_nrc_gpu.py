"""Radiance-cache MLP kernels against the NumPy reference (tests/nrc_reference.py).

Bars: the encoding to fp16 resolution; the forward pass to 2 % of the output
range (fp32 accumulation in a different order, fp16 activations); the loss
gradient per layer to 5 % in norm and 0.995 cosine similarity; one Adam
step to the reference update; and training that actually learns.
"""
import numpy as np
import pytest

import nrc_reference as ref
from gpugi_gb300 import nrc

pytestmark = pytest.mark.gpu

BOX_MIN, BOX_MAX = np.array([-1.0, 0.0, -1.0]), np.array([1.0, 2.0, 1.0])


def _queries(rng, n):
    q = np.concatenate([rng.uniform(BOX_MIN, BOX_MAX, (n, 3)), rng.normal(size=(n, 3)), rng.normal(size=(n, 3)),
                        rng.uniform(0.1, 0.9, (n, 3))], 1).astype(np.float32)
    q[:, 3:6] /= np.linalg.norm(q[:, 3:6], axis=1, keepdims=True)
    q[:, 6:9] /= np.linalg.norm(q[:, 6:9], axis=1, keepdims=True)
    return q


def _target(q):
    """A smooth radiance field to learn."""
    p = q[:, 0:3]
    return np.stack([1.0 + 0.5 * np.sin(3 * p[:, 0]) * q[:, 9], 0.8 + 0.4 * np.cos(2 * p[:, 1] + q[:, 4]),
                     0.5 + 0.3 * p[:, 2] * q[:, 11]], 1).astype(np.float32)


@pytest.fixture(scope="module")
def cache(cuda_ctx):
    c = nrc.RadianceCache(cuda_ctx, BOX_MIN, BOX_MAX, seed=3)
    yield c
    c.close()


def test_encoding_matches_reference(cuda_ctx, cache):
    import torch
    q = _queries(np.random.default_rng(1), 1000)
    enc = cache.encode(torch.from_numpy(q).cuda()).float().cpu().numpy()
    expect = ref.encode(q, BOX_MIN, BOX_MAX)
    assert np.abs(enc - expect).max() < 2e-3 * max(1.0, np.abs(expect).max())


def test_forward_matches_reference(cuda_ctx, cache):
    import torch
    rng = np.random.default_rng(2)
    q = _queries(rng, 4099)  # ragged tile count
    w = (rng.uniform(-1, 1, nrc.PARAMS) * 0.25).astype(np.float32)
    cache.set_weights(w)
    tq = torch.from_numpy(q).cuda()
    x0 = cache.encode(tq).cpu().numpy()
    _, out = ref.forward(x0, w)
    got = cache.infer(tq).cpu().numpy()
    expect = np.maximum(out[:, :3], 0)
    assert np.abs(got - expect).max() <= 0.02 * np.abs(expect).max() + 1e-3


@pytest.mark.parametrize("kernels,n", [("tcgen05", 3000), ("tcgen05", 40000), ("mma_sync", 3000)])
def test_gradient_matches_reference(cuda_ctx, cache, kernels, n):
    """Both training kernels: the tcgen05 one with fewer tiles than CTAs
    (3000 samples: 24 tiles, the last one partial) and with several tiles
    per CTA accumulating in tensor memory (40000 samples)."""
    import torch
    cache.set_kernels(kernels)
    rng = np.random.default_rng(3)
    q = _queries(rng, n)
    y = _target(q)
    w = (rng.uniform(-1, 1, nrc.PARAMS) * 0.2).astype(np.float32)
    cache.set_weights(w)
    samples = torch.from_numpy(np.concatenate([q, y], 1)).cuda()
    x0 = cache.encode(samples[:, :12].contiguous()).cpu().numpy()
    pred, grad, loss = cache.gradient(samples)
    rloss, rpred, rgrad = ref.loss_and_grad(x0, w, y)
    assert abs(loss / rloss - 1) < 0.02
    assert np.abs(pred - rpred).max() <= 0.02 * np.abs(rpred).max() + 1e-3
    for l, (i, o) in enumerate(ref.LAYER_SHAPES):
        a = grad[l * 4096: l * 4096 + i * o]
        b = rgrad[l * 4096: l * 4096 + i * o]
        rel = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-12)
        cos = float(a @ b) / max(np.linalg.norm(a) * np.linalg.norm(b), 1e-30)
        assert rel < 0.05 and cos > 0.995, (l, rel, cos)
    cache.set_kernels("tcgen05")


def test_training_kernels_agree(cuda_ctx):
    """The tcgen05 kernel and the mma.sync pair compute the same loss,
    predictions and gradient up to fp32 summation order (and the fp16
    roundings that order can flip)."""
    import torch
    rng = np.random.default_rng(8)
    n = 65536 + 77
    q = _queries(rng, n)
    samples = torch.from_numpy(np.concatenate([q, _target(q)], 1)).cuda()
    c = nrc.RadianceCache(cuda_ctx, BOX_MIN, BOX_MAX, seed=13)
    out = {}
    for k in ("mma_sync", "tcgen05"):
        c.set_kernels(k)
        out[k] = c.gradient(samples)
    (p0, g0, l0), (p1, g1, l1) = out["mma_sync"], out["tcgen05"]
    assert abs(l1 / l0 - 1) < 1e-3, (l0, l1)
    assert np.abs(p1 - p0).max() <= 1e-3 * np.abs(p0).max() + 1e-5
    for l, (i, o) in enumerate(ref.LAYER_SHAPES):
        a, b = g1[l * 4096: l * 4096 + i * o], g0[l * 4096: l * 4096 + i * o]
        rel = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-12)
        assert rel < 1e-2, (l, rel)
    assert cuda_ctx.device_error_bits() == 0
    c.close()


def test_tcgen05_wait_timeouts_are_reported_and_recoverable(cuda_ctx):
    """Every mbarrier wait of the tcgen05 kernels is bounded: with their MMAs
    and commits left out (gpugi_nrc_debug_stall, a barrier that nothing
    completes) the first wait of the inference and of the training kernel
    runs out after 20 ms; the call reports GPUGI_DEVERR_WAIT_TIMEOUT, the
    kernels free their tensor memory and end, and the next calls on the same
    context compute as before."""
    import re

    import torch
    from gpugi_gb300 import cuda
    rng = np.random.default_rng(9)
    q = _queries(rng, 4096)
    tq = torch.from_numpy(q).cuda()
    samples = torch.from_numpy(np.concatenate([q, _target(q)], 1)).cuda()
    c = nrc.RadianceCache(cuda_ctx, BOX_MIN, BOX_MAX, seed=21)
    c.set_kernels("tcgen05")
    before = c.infer(tq).cpu().numpy()
    _, g_before, l_before = c.gradient(samples)
    L = nrc._declare()

    def stalled_bits(call):
        try:
            call()
            return cuda_ctx.device_error_bits()
        except cuda.GpugiError as e:
            m = re.search(r"error bits (0x[0-9a-f]+)", str(e))
            assert e.status == 5 and m, str(e)
            return int(m.group(1), 16)

    cuda_ctx.check(L.gpugi_nrc_debug_stall(cuda_ctx.handle, c.handle, 1, 20_000_000))
    try:
        assert stalled_bits(lambda: c.infer(tq)) & 0x4
        assert stalled_bits(lambda: c.gradient(samples)) & 0x4
    finally:
        cuda_ctx.check(L.gpugi_nrc_debug_stall(cuda_ctx.handle, c.handle, 0, 0))
    assert cuda_ctx.device_error_bits() == 0
    assert np.array_equal(c.infer(tq).cpu().numpy(), before)
    _, g_after, l_after = c.gradient(samples)
    # the gradient sums run in a fixed order; the loss is summed with atomics
    assert np.array_equal(g_after, g_before) and abs(l_after / l_before - 1) < 1e-5
    assert cuda_ctx.device_error_bits() == 0
    c.close()


def test_adam_step_matches_reference(cuda_ctx, cache):
    import torch
    rng = np.random.default_rng(4)
    q = _queries(rng, 2048)
    samples = torch.from_numpy(np.concatenate([q, _target(q)], 1)).cuda()
    w0 = (rng.uniform(-1, 1, nrc.PARAMS) * 0.2).astype(np.float32)
    c = nrc.RadianceCache(cuda_ctx, BOX_MIN, BOX_MAX, seed=9, learning_rate=1e-2)
    c.set_weights(w0)
    _, g, _ = c.gradient(samples)
    c.train(samples)
    w1 = c.weights()
    m = 0.1 * g
    v = 0.01 * g * g
    expect = w0 - 1e-2 * (m / 0.1) / (np.sqrt(v / 0.01) + 1e-8)
    assert np.allclose(w1, expect, atol=1e-5, rtol=1e-3)
    c.close()


def test_training_learns_a_smooth_field(cuda_ctx):
    import torch
    rng = np.random.default_rng(5)
    c = nrc.RadianceCache(cuda_ctx, BOX_MIN, BOX_MAX, seed=11, learning_rate=1e-2)
    q_test = _queries(rng, 4096)
    y_test = _target(q_test)
    first = None
    for step in range(300):
        q = _queries(rng, 16384)
        loss = c.train(torch.from_numpy(np.concatenate([q, _target(q)], 1)).cuda())
        if first is None:
            first = loss
    pred = c.infer(torch.from_numpy(q_test).cuda()).cpu().numpy()
    rel = np.sqrt(((pred - y_test) ** 2).mean()) / np.sqrt((y_test ** 2).mean())
    assert loss < 0.1 * first, (first, loss)
    assert rel < 0.1, rel
    c.close()
