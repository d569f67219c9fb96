"""The C++ renderer classes (RendererSystem, Pathtracer, ..., TextureMSE)
through the headless driver, against the Python front end of the same C ABI.

The headless program sets up a RendererSystem the way the reference's
Application does; its first iteration uses the first light-sample set drawn from the
sampler state 123 and the frame seed of iteration 0, so the same images
come out of gpugi_render(samples=N, rngState=123).
"""
import json
import subprocess

import numpy as np
import pytest

from gpugi_gb300 import build, bvh, cuda, render, scenes

EXE = build.LIB / "gpugi_headless"


def _read_pfm(path):
    with open(path, "rb") as f:
        assert f.readline() == b"PF\n"
        w, h = map(int, f.readline().split())
        assert float(f.readline()) < 0
        return np.frombuffer(f.read(), dtype="<f4").reshape(h, w, 3)


def test_cli_rejects_bad_arguments(built):
    r = subprocess.run([str(EXE)], capture_output=True, text=True)
    assert r.returncode == 2 and "--scene is required" in r.stderr
    r = subprocess.run([str(EXE), "--scene", "x.bim", "--size", "0", "4"], capture_output=True, text=True)
    assert r.returncode == 2
    # waitMSE needs an MSE check interval, and the checks need a reference
    # image (the reference logs these cases as errors; here they are refused)
    r = subprocess.run([str(EXE), "--scene", "x.bim", "--wait-mse", "0.1"], capture_output=True, text=True)
    assert r.returncode == 2 and "--mse-check-interval" in r.stderr
    r = subprocess.run([str(EXE), "--scene", "x.bim", "--mse-check-interval", "2"], capture_output=True, text=True)
    assert r.returncode == 2 and "--reference" in r.stderr


@pytest.fixture(scope="module")
def room_file(tmp_path_factory, built):
    sc = scenes.cornell_room(seed=1, sphere_level=3, wall_grid=8)
    p = tmp_path_factory.mktemp("scene") / "room.bim"
    bvh.write_bvh_file(sc["positions"], sc["triangles"], str(p), normals=sc["normals"], texcoords=sc["texcoords"],
                       materials=sc["materials"], method="sweep", leaf_size=8)
    return sc, p


def _run(args):
    r = subprocess.run([str(EXE)] + [str(a) for a in args], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    return json.loads(r.stdout.strip().splitlines()[-1])


CAM = [0.0, 1.0, 3.4, 0.0, 1.0, 0.0, 40.0]


@pytest.mark.gpu
@pytest.mark.parametrize("renderer,pass_", [("Pathtracer", "PT"), ("BidirectionalPathtracer", "BPT"),
                                            ("LightPathtracer", "LT"), ("WhittedRayTracer", "WHITTED"),
                                            ("PhotonMapper", "PM"), ("PixelMapLighttracer", "IM"),
                                            ("HierarchyImportance", "HIERARCHY")])
def test_headless_matches_the_c_abi(cuda_ctx, room_file, tmp_path, renderer, pass_):
    sc, path = room_file
    W = H = 32
    iters = 4
    out = tmp_path / "out.pfm"
    info = _run(["--scene", path, "--renderer", renderer, "--size", W, H, "--camera", *CAM, "--iterations", iters,
                 "--path-length", 6, "--out", out])
    assert info["iterations"] == iters and info["renderer"] == renderer
    got = _read_pfm(out)

    b = bvh.read_bvh_file(str(path))
    ds = cuda_ctx.upload_scene(b, b.positions, cuda.vertex_info(b.normals, b.texcoords), b.materials)
    depth = 6
    if pass_ == "HIERARCHY":  # node NDFs from the file's approx_sggx chunk; the renderer's paths end at 4 vertices
        ds.set_hierarchy_ndf(b.sggx)
        depth = 4
    cam = render.camera_lookat(*scenes.CORNELL_CAMERA, W, H)
    img = render.Image(cuda_ctx, W, H)
    render.render(cuda_ctx, ds, cam, img, pass_, max_path_length=depth, samples=iters, rng_state=[123])
    expect = img.read()[..., :3] / iters
    if pass_ == "BPT":
        # eye paths pick light-cache entries by index, and the cache is
        # filled in atomic order: runs differ like independent samples
        assert abs(got.mean() / expect.mean() - 1) < 0.05, (got.mean(), expect.mean())
    else:
        # same seeds and light samples: equal up to float rounding in the
        # camera and normal encoding, which may divert a few paths
        close = np.abs(got - expect) <= 1e-4 * np.abs(expect).max() + 1e-6
        assert close.mean() > 0.97, close.mean()
        assert abs(got.mean() / expect.mean() - 1) < 0.02
    img.close()
    ds.close()


@pytest.mark.gpu
def test_headless_texture_mse_and_nrc(cuda_ctx, room_file, tmp_path):
    sc, path = room_file
    ref = tmp_path / "ref.pfm"
    common = ["--scene", path, "--size", 32, 32, "--camera", *CAM, "--path-length", 6]
    _run(common + ["--iterations", 8, "--out", ref])
    # the same run again, measured against the first: MSE ~ 0 (atomic order aside)
    info = _run(common + ["--iterations", 8, "--reference", ref])
    assert 0.0 <= info["mse"] < 1e-9
    # a shorter run is noisier
    info4 = _run(common + ["--iterations", 2, "--reference", ref])
    assert info4["mse"] > 1e-6
    for renderer in ("NrcPathtracer", "NrcBidirectionalPathtracer"):
        nrc = tmp_path / f"{renderer}.pfm"
        info_nrc = _run(common + ["--renderer", renderer, "--iterations", 8, "--out", nrc])
        assert info_nrc["renderer"] == renderer
        img = _read_pfm(nrc)
        assert np.isfinite(img).all() and img.mean() > 0


@pytest.mark.gpu
def test_headless_mse_checks_and_wait_mse(cuda_ctx, room_file, tmp_path):
    """--mse-check-interval prints the MSE against the reference every N
    iterations (Application::MSEChecks); --wait-mse stops at the first check
    below the goal (the script command waitMSE), well before the cap."""
    sc, path = room_file
    ref = tmp_path / "ref.pfm"
    common = ["--scene", path, "--size", 32, 32, "--camera", *CAM, "--path-length", 6]
    _run(common + ["--iterations", 256, "--out", ref])
    r = subprocess.run([str(EXE)] + [str(a) for a in common + ["--iterations", 12, "--reference", ref,
                                                                  "--mse-check-interval", 4]],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    lines = [json.loads(x) for x in r.stdout.strip().splitlines()]
    checks, summary = lines[:-1], lines[-1]
    assert [c["iteration"] for c in checks] == [4, 8, 12]
    assert checks[-1]["mse"] == pytest.approx(summary["mse"], rel=1e-6)
    assert checks[0]["mse"] > checks[-1]["mse"] > 0
    goal = 0.5 * (checks[0]["mse"] + checks[-1]["mse"])  # between the 4- and the 12-iteration MSE
    r = subprocess.run([str(EXE)] + [str(a) for a in common + ["--iterations", 200, "--reference", ref,
                                                                  "--mse-check-interval", 2, "--wait-mse", goal]],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    lines = [json.loads(x) for x in r.stdout.strip().splitlines()]
    checks, summary = lines[:-1], lines[-1]
    assert summary["reached"] is True and summary["mse_nan"] is False
    assert summary["iterations"] == summary["reached_iteration"] == checks[-1]["iteration"] < 200
    assert checks[-1]["mse"] < goal and all(c["mse"] >= goal for c in checks[:-1])
    assert summary["reached_wall_ms"] > 0


@pytest.mark.gpu
def test_headless_reads_materials_from_scene_json(cuda_ctx, room_file, tmp_path):
    """A scene file with material names and a gpugi-style scene JSON beside
    it renders like the same file carrying the material records."""
    sc, path = room_file
    mats = sc["materials"].reshape(-1, 24)
    names = [f"mat{i}" for i in range(mats.shape[0])]
    entries = {n: {"type": "legacy", "albedo": [float(x) for x in m[0:3]], "specularColor": [0, 0, 0],
                   "roughness": [1], "opacity": [1], "emissivity": [float(x) for x in m[12:15]]}
               for n, m in zip(names, mats)}
    named = tmp_path / "named.bim"
    bvh.write_bvh_file(sc["positions"], sc["triangles"], str(named), normals=sc["normals"],
                       texcoords=sc["texcoords"], material_names=names, method="sweep", leaf_size=8)
    (tmp_path / "named.json").write_text(json.dumps({"scene": "named.bim", "materials": entries}))
    assert np.allclose(bvh.materials_from_json((tmp_path / "named.json").read_text(), names), mats)
    common = ["--size", 32, 32, "--camera", *CAM, "--path-length", 6, "--iterations", 4]
    a, b_ = tmp_path / "a.pfm", tmp_path / "b.pfm"
    _run(["--scene", path] + common + ["--out", a])
    _run(["--scene", named] + common + ["--out", b_])
    ia, ib = _read_pfm(a), _read_pfm(b_)
    assert np.abs(ia - ib).max() <= 1e-5 * np.abs(ia).max() + 1e-6


@pytest.mark.gpu
@pytest.mark.parametrize("renderer", ["Pathtracer", "LightPathtracer", "BidirectionalPathtracer"])
def test_headless_checkpoint_resume_continues_the_estimator(cuda_ctx, room_file, tmp_path, renderer):
    """8 iterations in one run equal 5 iterations, a checkpoint, and 3 more
    iterations in a second run that resumes it (same frame indices, same
    light-sample sets; the sums differ only by the order of the atomic
    additions; BPT's eye paths pick light-cache entries by index from a
    cache filled in atomic order, so there the runs agree in the mean).
    The checkpoint's files are the documented format."""
    from gpugi_gb300 import checkpoint
    sc, path = room_file
    base = ["--scene", str(path), "--renderer", renderer, "--size", 24, 20, "--camera", *CAM]
    one = _run(base + ["--iterations", 8, "--out", tmp_path / "one.pfm"])
    ck = tmp_path / "ck"
    first = _run(base + ["--iterations", 5, "--checkpoint", ck])
    side, rgba, rgb64 = checkpoint.read(str(ck))
    assert side["iterations"] == side["next_iteration"] == 5 and side["renderer"] == first["renderer"]
    assert rgb64 is None and rgba.shape == (20, 24, 4)
    assert np.allclose(checkpoint.read_pfm(str(ck) + ".pfm"), rgba[..., :3] / 5, rtol=1e-6, atol=0)
    two = _run(base + ["--resume", ck, "--iterations", 3, "--out", tmp_path / "two.pfm"])
    assert two["iterations"] == one["iterations"] == 8
    a, b = _read_pfm(tmp_path / "one.pfm"), _read_pfm(tmp_path / "two.pfm")
    if renderer == "BidirectionalPathtracer":
        assert abs(b.mean() / a.mean() - 1) < 0.05, (a.mean(), b.mean())
    else:
        assert np.abs(a - b).max() <= 1e-5 * np.abs(a).max() + 1e-7
    # a checkpoint of another renderer or size is refused
    other = "Pathtracer" if renderer != "Pathtracer" else "LightPathtracer"
    r = subprocess.run([str(EXE), "--scene", str(path), "--renderer", other, "--size", "24", "20", "--resume", str(ck)],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 1 and "checkpoint of renderer" in r.stderr
