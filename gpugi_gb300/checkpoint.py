"""Checkpoint and resume of a long accumulation.

The reference only saves the normalised backbuffer as PFM
(Application::SaveImage, gpugi/application.cpp:394-414; WritePfm,
gpugi/imageut/hdrimage.cpp:6-33). A checkpoint keeps that image and adds what
resuming needs, so that a render split over several runs accumulates the same
estimator as one run (equal up to the order of the atomic sums):

  <base>.pfm    the average (sums / iterations), RGB, rows bottom-up: what
                SaveImage writes
  <base>.accum  the exact sums: height x width x 4 float32 (RGBA, row 0 at the
                bottom), then height x width x 3 float64 when the image has an
                FP64 accumulation; little-endian, no header
  <base>.json   the sidecar: format, version, width, height, fp64, iterations
                (the divisor of the sums), next_iteration (the frame index of
                the next iteration: it seeds the per-pixel random streams),
                rng_state (the light sampler's state that draws the next
                iteration's light samples) and the render settings
                (pass, max_path_length, rr_start_depth, random, sky)

The C++ renderer (RendererSystem::SaveCheckpoint / LoadCheckpoint) writes
and reads the same files.
"""
from __future__ import annotations

import json
import os

import numpy as np

FORMAT = "gpugi_gb300 checkpoint"
VERSION = 1


def write_pfm(path: str, rgb: np.ndarray) -> None:
    """RGB PFM, little-endian (scale -1), rows in array order (row 0 is the
    file's first row, the bottom of the image)."""
    rgb = np.ascontiguousarray(rgb, dtype="<f4")
    h, w = rgb.shape[:2]
    with open(path, "wb") as f:
        f.write(b"PF\n%d %d\n-1.0\n" % (w, h))
        f.write(rgb.tobytes())


def read_pfm(path: str) -> np.ndarray:
    with open(path, "rb") as f:
        kind = f.readline().strip()
        if kind not in (b"PF", b"Pf"):
            raise ValueError(f"{path}: not a PFM file")
        w, h = (int(x) for x in f.readline().split())
        scale = float(f.readline())
        data = np.frombuffer(f.read(), dtype="<f4" if scale < 0 else ">f4")
    c = 3 if kind == b"PF" else 1
    if data.size != w * h * c:
        raise ValueError(f"{path}: {data.size} values, expected {w * h * c}")
    return data.reshape(h, w, c).astype(np.float32)


def write(base: str, rgba: np.ndarray, rgb64: np.ndarray | None, iterations: int, next_iteration: int,
          rng_state: int, **settings) -> None:
    """Write a checkpoint from host copies of the sums."""
    h, w = rgba.shape[:2]
    write_pfm(base + ".pfm", rgba[..., :3] / max(iterations, 1))
    with open(base + ".accum", "wb") as f:
        f.write(np.ascontiguousarray(rgba, dtype="<f4").tobytes())
        if rgb64 is not None:
            f.write(np.ascontiguousarray(rgb64, dtype="<f8").tobytes())
    side = {"format": FORMAT, "version": VERSION, "width": w, "height": h, "fp64": rgb64 is not None,
            "iterations": int(iterations), "next_iteration": int(next_iteration), "rng_state": int(rng_state),
            "image": os.path.basename(base) + ".pfm", "accumulation": os.path.basename(base) + ".accum"}
    side.update(settings)
    with open(base + ".json", "w") as f:
        json.dump(side, f, indent=1)
        f.write("\n")


def read(base: str) -> tuple[dict, np.ndarray, np.ndarray | None]:
    """(sidecar, rgba sums, rgb64 sums or None)."""
    with open(base + ".json") as f:
        side = json.load(f)
    if side.get("format") != FORMAT or side.get("version") != VERSION:
        raise ValueError(f"{base}.json: not a version-{VERSION} checkpoint")
    h, w = int(side["height"]), int(side["width"])
    raw = open(os.path.join(os.path.dirname(base), side["accumulation"]), "rb").read()
    n32 = h * w * 4 * 4
    n64 = h * w * 3 * 8 if side["fp64"] else 0
    if len(raw) != n32 + n64:
        raise ValueError(f"{base}.accum: {len(raw)} bytes, expected {n32 + n64}")
    rgba = np.frombuffer(raw[:n32], dtype="<f4").reshape(h, w, 4).astype(np.float32)
    rgb64 = np.frombuffer(raw[n32:], dtype="<f8").reshape(h, w, 3).astype(np.float64) if n64 else None
    return side, rgba, rgb64


def save(base: str, image, iterations: int, next_iteration: int, rng_state: int, **settings) -> None:
    """Checkpoint a render.Image after `iterations` accumulated iterations."""
    write(base, image.read(), image.read64() if image.fp64 else None, iterations, next_iteration, rng_state,
          **settings)


def load(base: str, image) -> dict:
    """Restore the sums of a checkpoint into a render.Image of the same size
    (and FP64 flag) and return the sidecar; continue with
    iteration=side["next_iteration"] and rng_state=[side["rng_state"]]."""
    side, rgba, rgb64 = read(base)
    if (image.width, image.height) != (side["width"], side["height"]) or image.fp64 != side["fp64"]:
        raise ValueError("checkpoint size or FP64 flag differs from the image")
    image.write(rgba, rgb64)
    return side
