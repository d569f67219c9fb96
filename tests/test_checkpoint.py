"""Checkpoint files (gpugi_gb300.checkpoint) on the CPU: the PFM writer and
reader, and the exact round trip of the sums and the sidecar."""
import json

import numpy as np
import pytest

from gpugi_gb300 import checkpoint


def test_pfm_round_trip(tmp_path):
    rgb = np.random.default_rng(1).standard_normal((5, 7, 3)).astype(np.float32)
    p = str(tmp_path / "x.pfm")
    checkpoint.write_pfm(p, rgb)
    raw = open(p, "rb").read()
    assert raw.startswith(b"PF\n7 5\n-1.0\n") and len(raw) == len(b"PF\n7 5\n-1.0\n") + rgb.size * 4
    assert np.array_equal(checkpoint.read_pfm(p), rgb)


@pytest.mark.parametrize("fp64", [False, True])
def test_sums_and_sidecar_round_trip_exactly(tmp_path, fp64):
    g = np.random.default_rng(2)
    rgba = (g.random((6, 9, 4)) * 100).astype(np.float32)
    rgb64 = g.random((6, 9, 3)) * 100 if fp64 else None
    base = str(tmp_path / "ck")
    checkpoint.write(base, rgba, rgb64, iterations=37, next_iteration=1037, rng_state=2**64 - 5, pass_name="PT",
                     max_path_length=8, sky=[0.5, 0.5, 0.5])
    side, a, b = checkpoint.read(base)
    assert np.array_equal(a, rgba)
    assert (b is None) if not fp64 else np.array_equal(b, rgb64)
    assert side["iterations"] == 37 and side["next_iteration"] == 1037 and side["rng_state"] == 2**64 - 5
    assert side["width"] == 9 and side["height"] == 6 and side["fp64"] == fp64 and side["pass_name"] == "PT"
    assert np.allclose(checkpoint.read_pfm(base + ".pfm"), rgba[..., :3] / 37, rtol=1e-6)


def test_damaged_checkpoints_are_refused(tmp_path):
    base = str(tmp_path / "ck")
    checkpoint.write(base, np.zeros((2, 3, 4), np.float32), None, 1, 1, 123)
    with open(base + ".accum", "ab") as f:
        f.write(b"x")
    with pytest.raises(ValueError, match="bytes"):
        checkpoint.read(base)
    side = json.load(open(base + ".json"))
    side["version"] = 99
    json.dump(side, open(base + ".json", "w"))
    with pytest.raises(ValueError, match="version"):
        checkpoint.read(base)
