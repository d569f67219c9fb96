"""Build recipe of oracle/_ref: the reference's own shader text compiled as C++.

ORACLE — test infrastructure only. gpugi's hot path exists only as GLSL
compute shaders (gpugi/shader/), which need an OpenGL 4.5 context that no
machine here has. Their text is nearly C++ already, so this recipe rewrites
it mechanically and compiles it on the CPU against oracle/ref_shim.hpp (the
GLSL built-ins). The library it builds, oracle/_ref/libgpugi_ref.so, is the
reference's own code for the path (traversal, the random and helper
functions, pathtracer.comp, lighttracer.comp with and without
SAVE_LIGHT_CACHE, showlightcaches.comp, pathtracer_bidir.comp,
whittedraytracer.comp, the photon mapper's photondistribution.comp and
gather.comp, the importon map light tracer's importondistribution.comp
and photontracing.comp, both with the lossless hash map, and the hierarchy
renderer's hierarchypathtracer.comp, acquisition2.comp, propagation and
node-material passes);
tests/test_ref_pinned.py checks the oracle's restatement (oracle/*.cpp)
against it bit for bit.

The rewrite (nothing else is changed; no reference text is stored in the
repository: the rewritten copies live in oracle/_ref/gen/, which is
git-ignored and rebuilt from the reference tree):
  * `#version` / `#extension` lines are dropped; `#include "x"` becomes
    `#include "x.h"` (the rewritten copy);
  * `layout(...)` qualifiers and the storage words `uniform`, `buffer`,
    `restrict`, `readonly`, `writeonly`, `coherent`, `volatile` are dropped;
    the members of a uniform or storage block become globals (GLSL puts
    them in global scope too); an unsized array member becomes a pointer;
    the compute shader's `in;` local-size statement is dropped;
  * parameter qualifiers: `out T x` and `inout T x` become `T& x`, `in` is
    dropped;
  * floating literals get an `f` suffix (GLSL literals are single precision);
  * multi-component swizzle reads (`.xyz`, `.xx`, `.yz` ...) become calls of
    the shim's swizzle functions;
  * vector constructors `vecN(a, b)` become `vecN{a, b}`: GLSL evaluates
    arguments left to right (random.glsl:48, `vec2(Random(seed),
    Random(seed))`, depends on it), C++ only inside braces;
  * `#define TRIANGLES_PER_LEAF 2` (scenedata.glsl:5, the Bim library's leaf
    size) becomes a default the build overrides with the scene's leaf size
    (bvhmake writes 8), as the shader's other compile-time constants are
    injected; MAX_PATHLENGTH, which the application injects, reads a global.

Run: python oracle/ref_build.py [--reference DIR] [--force]. Needs g++ and
the reference tree; without the tree there is nothing to build and the
pinned tests skip.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT_DIR = HERE / "_ref"
GEN = OUT_DIR / "gen"
LIB = OUT_DIR / "libgpugi_ref.so"
DEFAULT_REFERENCE = Path(os.environ.get("GPUGI_REFERENCE", "/root/reference")) / "gpugi" / "shader"

# Shader files the glue includes (directly or through #include).
FILES = ["helper.glsl", "scenedata.glsl", "intersectiontests.glsl", "random.glsl", "traceray.glsl",
         "globaluniforms.glsl", "materials.glsl", "lightsource.glsl", "stdheader.glsl", "pathtracer.comp",
         "lighttracer.comp", "screenreproject.glsl", "showlightcaches.comp", "bidirpathtracer/lightcache.glsl",
         "bidirpathtracer/pathtracer_bidir.comp", "whittedraytracer.comp", "photonmapper/photondistribution.comp",
         "photonmapper/gather.comp", "photonmapper/photonmap.glsl", "maps/hashmap.glsl", "maps/grid.glsl",
         "pixelmaplt/importondistribution.comp", "pixelmaplt/photontracing.comp", "pixelmaplt/importonmap.glsl",
         "hierarchy/hierarchypathtracer.comp", "hierarchy/sggx.glsl", "hierarchy/acquisition2.comp",
         "hierarchy/counthits.glsl", "hierarchy/importanceubo.glsl", "hierarchy/hierarchypropagation_init.comp",
         "hierarchy/hierarchypropagation_nodes.comp", "hierarchy/hierarchymaterialbuffer.glsl",
         "hierarchy/sampleleafmaterials.comp", "hierarchy/pullmaterials.comp"]
OVERRIDABLE = {"TRIANGLES_PER_LEAF"}

_CTOR = re.compile(r"\b((?:i|u|b)?vec[234])\s*\(")


def brace_constructors(t: str) -> str:
    out, i = [], 0
    while True:
        m = _CTOR.search(t, i)
        if not m:
            out.append(t[i:])
            return "".join(out)
        out.append(t[i:m.start()])
        depth, j = 1, m.end()
        while depth:
            depth += {"(": 1, ")": -1}.get(t[j], 0)
            j += 1
        out.append(m.group(1) + "{" + brace_constructors(t[m.end():j - 1]) + "}")
        i = j


_FLOAT = re.compile(r"(?<![\w.])((?:\d+\.\d*|\.\d+)(?:[eE][+-]?\d+)?|\d+[eE][+-]?\d+)(?![\w.])")
_SWIZZLE = re.compile(r"\.([xyzwrgba]{2,4})\b(?!\s*\()")


def rewrite(text: str) -> str:
    out = []
    for line in text.splitlines():
        s = line.strip()
        if s.startswith("#version") or s.startswith("#extension"):
            continue
        m = re.match(r'\s*#\s*include\s+"([^"]+)"', line)
        if m:
            out.append('#include "%s.h"' % m.group(1))
            continue
        m = re.match(r"\s*#\s*define\s+(\w+)\s+(.*)$", line)
        if m and m.group(1) in OVERRIDABLE:
            out.append("#ifndef %s\n#define %s %s\n#endif" % (m.group(1), m.group(1), m.group(2)))
            continue
        out.append(line)
    t = "\n".join(out) + "\n"
    # layout qualifiers and storage words
    t = re.sub(r"\blayout\s*\([^)]*\)\s*", "", t)
    t = re.sub(r"\b(?:uniform|buffer)\s+\w+\s*\{(.*?)\}\s*;", r"\1", t, flags=re.S)
    t = re.sub(r"\b(?:uniform|restrict|readonly|writeonly|coherent|volatile)\s+", "", t)
    t = re.sub(r"^\s*in\s*;", "", t, flags=re.M)
    t = re.sub(r"(\b\w+)\s+(\w+)\s*\[\s*\]\s*;", r"\1* \2;", t)
    # parameter qualifiers
    t = re.sub(r"\b(?:inout|out)\s+((?:const\s+)?\w+)\s+(\w+)", r"\1& \2", t)
    t = re.sub(r"\bin\s+(?=\w+\s+\w+)", "", t)
    # literals and swizzles (comments are rewritten too; harmless)
    t = _FLOAT.sub(lambda m: m.group(1) + "f", t)
    t = _SWIZZLE.sub(lambda m: ".%s()" % m.group(1), t)
    return brace_constructors(t)


def generate(reference: Path) -> None:
    GEN.mkdir(parents=True, exist_ok=True)
    for name in FILES:
        src = reference / name
        dst = GEN / (name + ".h")
        dst.parent.mkdir(parents=True, exist_ok=True)
        dst.write_text("// rewritten from the reference's %s by oracle/ref_build.py (not stored in the repository)\n"
                       % name + rewrite(src.read_text(encoding="utf-8", errors="replace")))


def build(reference: Path | None = None, force: bool = False) -> Path | None:
    """Rewrite the shaders (when the reference tree is present) and compile.
    Without the tree, rewritten copies already in oracle/_ref/gen/ (made on a
    machine that has it) are compiled as they are; without either there is
    nothing to build and None is returned."""
    ref = Path(reference) if reference else DEFAULT_REFERENCE
    have_tree = ref.is_dir()
    have_gen = all((GEN / (f + ".h")).exists() for f in FILES)
    if not have_tree and not have_gen:
        return LIB if LIB.exists() else None
    srcs = [ref / f for f in FILES] if have_tree else [GEN / (f + ".h") for f in FILES]
    deps = [HERE / "ref_shim.hpp", HERE / "ref_glue.cpp", Path(__file__)] + srcs
    if not force and LIB.exists() and all(d.stat().st_mtime <= LIB.stat().st_mtime for d in deps):
        return LIB
    if have_tree:
        generate(ref)
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-shared", "-w",
           "-Wno-narrowing",
           "-I", str(GEN), "-I", str(HERE), "-o", str(LIB), str(HERE / "ref_glue.cpp"), "-pthread"]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle/_ref build failed:\n" + r.stdout[-6000:])
    return LIB


if __name__ == "__main__":
    args = sys.argv[1:]
    refdir = None
    if "--reference" in args:
        refdir = Path(args[args.index("--reference") + 1])
    print(build(refdir, force="--force" in args))
