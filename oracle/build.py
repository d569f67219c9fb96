"""Build recipe for the oracle (test infrastructure only).

Compiles the C++ restatement of gpugi's shaders into oracle/lib/liboracle.so.
-ffp-contract=off keeps FMA contraction out on both x86 and Arm, so the
oracle's float arithmetic is the plain IEEE sequence written in the source.
The reference itself cannot be compiled (its shaders need OpenGL, its host
code needs the missing epsilon/bim/glhelper submodules), so there is no
oracle/_ref build.
"""
from __future__ import annotations

import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
SOURCES = ["trace.cpp", "render.cpp", "lights.cpp"]
OUT = HERE / "lib" / "liboracle.so"


def build(force: bool = False) -> Path:
    OUT.parent.mkdir(parents=True, exist_ok=True)
    srcs = [HERE / s for s in SOURCES if (HERE / s).exists()]
    deps = srcs + list(HERE.glob("*.hpp"))
    if not force and OUT.exists() and all(d.stat().st_mtime <= OUT.stat().st_mtime for d in deps):
        return OUT
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-shared",
           "-o", str(OUT)] + [str(s) for s in srcs] + ["-pthread"]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
