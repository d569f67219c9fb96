"""The bounds-checked library (libgpugi_cuda_checked.so: the same sources
compiled with -DGPUGI_CHECKED=1, node, leaf-slot, vertex and material
indexes checked before every fetch). On valid scenes it returns the
oracle's results in every trace mode and renders the passes with no error
bit; when a walk reaches a node at or past a lowered node limit
(gpugi_debug_limit_nodes: the node array itself is unchanged, so every fetch
stays inside it) the call fails with GPUGI_DEVERR_BOUNDS. The checks run in
a child process that loads the checked library (GPUGI_CHECKED=1)."""
import os
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent

CHILD = r'''
import re

import numpy as np

import oracle
from gpugi_gb300 import bvh, cuda, render, scenes

L = cuda.lib()
assert L.gpugi_version().endswith(b"checked"), L.gpugi_version()
ctx = cuda.Context()
sc = scenes.displaced_icosphere(65536, seed=1)
b = bvh.build_bvh(sc["positions"], sc["triangles"], method="sweep")
ds = ctx.upload_scene(b, sc["positions"])
rays = scenes.aimed_rays(1 << 16, sc["positions"], seed=5, spread=2.5)
o = oracle.trace_closest(b, sc["positions"], rays)
oa = oracle.trace_any(b, sc["positions"], rays)["occluded"]
bits = lambda a: np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)
for mode in range(6):
    ctx.set_trace_config(mode=mode)
    g = cuda.trace_closest(ctx, ds, rays)
    assert np.array_equal(g["slot"], o["slot"]), mode
    assert np.array_equal(bits(g["t"]), bits(o["t"])), mode
    hit = o["slot"] >= 0
    assert np.array_equal(bits(g["u"])[hit], bits(o["u"])[hit]), mode
    assert np.array_equal(bits(g["v"])[hit], bits(o["v"])[hit]), mode
    assert np.array_equal(cuda.trace_any(ctx, ds, rays), oa), mode
assert ctx.device_error_bits() == 0

# walks that reach a node past the lowered limit end with the bounds bit
ctx.check(L.gpugi_debug_limit_nodes(ds.handle, b.num_nodes // 2))
for mode in range(6):
    ctx.set_trace_config(mode=mode)
    for any_hit in (False, True):
        try:
            (cuda.trace_any if any_hit else cuda.trace_closest)(ctx, ds, rays)
        except cuda.GpugiError as e:
            m = re.search(r"error bits (0x[0-9a-f]+)", str(e))
            assert e.status == 5 and m and int(m.group(1), 16) & 0x20, (mode, any_hit, str(e))
        else:
            raise AssertionError(f"mode {mode} any_hit {any_hit}: no bounds error")
ctx.check(L.gpugi_debug_limit_nodes(ds.handle, 0))
ctx.set_trace_config(mode=3)
g = cuda.trace_closest(ctx, ds, rays)
assert np.array_equal(g["slot"], o["slot"]) and ctx.device_error_bits() == 0
ds.close()

# the passes shade through the checked vertex and material fetches
room = scenes.cornell_room(seed=1, sphere_level=3, wall_grid=8)
rb = bvh.build_bvh(room["positions"], room["triangles"], method="sweep")
rs = ctx.upload_scene(rb, room["positions"], cuda.vertex_info(room["normals"], room["texcoords"]),
                      room["materials"])
cam = render.camera_lookat(*scenes.CORNELL_CAMERA, 64, 48)
for pass_ in ("PT", "LT", "BPT"):
    img = render.Image(ctx, 64, 48)
    render.render(ctx, rs, cam, img, pass_, max_path_length=6, samples=4, rng_state=[3])
    a = img.read()
    assert np.isfinite(a).all() and a[..., :3].mean() > 0, pass_
    assert ctx.device_error_bits() == 0, pass_
    img.close()
rs.close()
print("checked library ok")
'''


@pytest.mark.gpu
def test_checked_library(tmp_path):
    lib = ROOT / "gpugi_gb300" / "lib" / "libgpugi_cuda_checked.so"
    assert lib.exists(), "the checked library is built with the others (python -m gpugi_gb300.build)"
    script = tmp_path / "checked_child.py"
    script.write_text(CHILD)
    env = dict(os.environ, GPUGI_CHECKED="1", PYTHONPATH=str(ROOT))
    r = subprocess.run([sys.executable, str(script)], cwd=ROOT, env=env, capture_output=True, text=True,
                       timeout=900)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    assert "checked library ok" in r.stdout
