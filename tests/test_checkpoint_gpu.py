"""Resuming a checkpointed render through the Python API: 8 iterations in
one call equal 5 iterations, a checkpoint written and read back into a new
image, and 3 more iterations from the checkpoint's frame index and light
sampler state (up to the order of the atomic sums)."""
import numpy as np
import pytest

from gpugi_gb300 import bvh, checkpoint, cuda, render, scenes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("pass_", ["PT", "LT"])
def test_resume_continues_the_estimator(cuda_ctx, tmp_path, pass_):
    sc = scenes.cornell_room(seed=1, sphere_level=3, wall_grid=8)
    b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep")
    ds = cuda_ctx.upload_scene(b, sc["positions"], cuda.vertex_info(sc["normals"], sc["texcoords"]), sc["materials"])
    W, H = 40, 32
    cam = render.camera_lookat(*scenes.CORNELL_CAMERA, W, H)
    opts = dict(max_path_length=6, num_light_samples=render.DEFAULT_LIGHT_SAMPLES[pass_])
    full = render.Image(cuda_ctx, W, H, fp64=True)
    render.render(cuda_ctx, ds, cam, full, pass_, samples=8, iteration=0, rng_state=[5], **opts)

    part = render.Image(cuda_ctx, W, H, fp64=True)
    st = [5]
    render.render(cuda_ctx, ds, cam, part, pass_, samples=5, iteration=0, rng_state=st, **opts)
    base = str(tmp_path / "ck")
    checkpoint.save(base, part, iterations=5, next_iteration=5, rng_state=st[0], pass_name=pass_)
    part.close()

    resumed = render.Image(cuda_ctx, W, H, fp64=True)
    side = checkpoint.load(base, resumed)
    st2 = [side["rng_state"]]
    render.render(cuda_ctx, ds, cam, resumed, pass_, samples=3, iteration=side["next_iteration"], rng_state=st2,
                  **opts)
    a, c = full.read64(), resumed.read64()
    assert np.abs(a - c).max() <= 1e-9 * np.abs(a).max()
    assert np.abs(full.read() - resumed.read()).max() <= 1e-5 * np.abs(full.read()).max()
    with pytest.raises(ValueError):
        checkpoint.load(base, render.Image(cuda_ctx, W + 1, H, fp64=True))
    for x in (full, resumed, ds):
        x.close()
