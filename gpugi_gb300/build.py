"""Build recipe for the native libraries of gpugi_gb300 (no cmake).

  lib/libgpugi_bvhmake.so   host C++ BVH builder (bvhmake restatement)
  lib/libgpugi_cuda.so      sm_103a kernels + the C ABI of include/gpugi_cuda.h
  lib/gpugi_headless        headless driver over the C++ Renderer classes

Everything is compiled in-tree and in parallel; nvcc targets sm_103a only.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
LIB = PKG / "lib"
OBJ = PKG / "lib" / "obj"
INCLUDE = ROOT / "include"

NVCC = os.environ.get("NVCC", shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc")
CXX = os.environ.get("CXX", "g++")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# No FMA contraction in host code: the builder's float arithmetic must not
# depend on the compiler's contraction default, which differs between x86 and Arm.
HOST_FLAGS = ["-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off", "--expt-relaxed-constexpr",
              "-I", str(INCLUDE), "-I", str(CSRC)] + ARCH

# extra nvcc arguments (for example -D settings of the kernels), from the environment
NVCC_FLAGS += os.environ.get("GPUGI_NVCC_EXTRA", "").split()

CUDA_SOURCES = ["trace.cu", "scene.cu", "render.cu", "capi.cu", "host.cu", "noalloc.cu", "nrc.cu", "tune.cu", "build.cu",
                "hierarchy.cu"]


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(map(str, cmd)) + "\n" + r.stdout)
    return r.stdout


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def _headers():
    return list(CSRC.rglob("*.cuh")) + list(CSRC.rglob("*.hpp")) + list(INCLUDE.glob("*.h"))


def build_bvhmake(force=False) -> Path:
    LIB.mkdir(parents=True, exist_ok=True)
    out = LIB / "libgpugi_bvhmake.so"
    srcs = [CSRC / "bvhmake" / "bvhmake.cpp", CSRC / "bvhmake" / "material_json.cpp"]
    if force or _stale(out, srcs + _headers()):
        _run([CXX] + HOST_FLAGS + ["-shared", "-o", str(out)] + [str(s) for s in srcs] + ["-pthread"])
    return out


def build_cuda(force=False, jobs=None, checked=False) -> Path:
    """libgpugi_cuda.so, or with checked=True libgpugi_cuda_checked.so: the
    same sources compiled with -DGPUGI_CHECKED=1 (device indexes checked
    before every node, slot, vertex and material fetch; a bad one sets
    GPUGI_DEVERR_BOUNDS and the fetch is skipped)."""
    out = LIB / ("libgpugi_cuda_checked.so" if checked else "libgpugi_cuda.so")
    obj = OBJ / "checked" if checked else OBJ
    obj.mkdir(parents=True, exist_ok=True)
    flags = NVCC_FLAGS + (["-DGPUGI_CHECKED=1"] if checked else [])
    srcs = [CSRC / s for s in CUDA_SOURCES if (CSRC / s).exists()]
    hdrs = _headers()
    objs = []
    todo = []
    for s in srcs:
        o = obj / (s.stem + ".o")
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            todo.append([NVCC] + flags + ["-c", str(s), "-o", str(o)])
    with cf.ThreadPoolExecutor(max_workers=jobs or max(1, len(todo))) as ex:
        list(ex.map(_run, todo))
    if force or todo or _stale(out, objs):
        _run([NVCC] + ARCH + ["-shared", "-o", str(out)] + [str(o) for o in objs] + ["-lcudart"])
    return out


def build_headless(force=False) -> Path | None:
    src_dir = CSRC / "host"
    if not src_dir.exists():
        return None
    out = LIB / "gpugi_headless"
    srcs = sorted(src_dir.glob("*.cpp"))
    deps = srcs + _headers() + [LIB / "libgpugi_cuda.so", LIB / "libgpugi_bvhmake.so"]
    if force or _stale(out, deps):
        _run([CXX] + HOST_FLAGS + ["-I", str(INCLUDE), "-I", str(src_dir), "-o", str(out)] + [str(s) for s in srcs]
             + ["-L", str(LIB), "-lgpugi_cuda", "-lgpugi_bvhmake", "-Wl,-rpath,$ORIGIN", "-pthread"])
    return out


def build_all(force=False):
    LIB.mkdir(parents=True, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=3) as ex:
        f1 = ex.submit(build_bvhmake, force)
        f2 = ex.submit(build_cuda, force)
        f3 = ex.submit(build_cuda, force, None, True)
        f1.result()
        f2.result()
        f3.result()
    build_headless(force)


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
    print("built", sorted(p.name for p in LIB.iterdir() if p.is_file()))
