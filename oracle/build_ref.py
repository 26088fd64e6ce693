"""Build recipe for oracle/_ref/libref_shaders.so (test infrastructure).

Compiles the reference's own shader sources -- res/billboard_vert_instanced.glsl,
res/first_voxelize.glsl, res/second_voxelize.glsl and res/conetrace_frag.glsl
of jaafersheriff/Cloud-Renderer, read where they lie in the reference checkout
(CLOUD_RENDERER_REFERENCE; by default its mount in the build container) --
as C++ through oracle/ref_shim/glsl_shim.hpp, together with the driver
oracle/ref_shim/ref_driver.inc that runs them the way the reference's host
code does.  The translation unit is assembled in memory and piped to g++:
each shader's text goes into its own namespace, its `#version` line blanked
and its `inout` parameters written as C++ references;
no copy of a reference source is written anywhere.  The output (and only it)
goes to oracle/_ref/, which git ignores.

The library exists only where the reference is present; tests that need it
skip otherwise, and the fixtures under tests/golden/ (made from it by
tests/golden/make_golden.py) carry its results everywhere else.
"""
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference checkout: CLOUD_RENDERER_REFERENCE, else its mount in the
# build container
REFERENCE = os.environ.get("CLOUD_RENDERER_REFERENCE", "/root/reference")
SHIM = os.path.join(HERE, "ref_shim")
OUT_DIR = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT_DIR, "libref_shaders.so")
SHADERS = [
    ("ref_vert", "res/billboard_vert_instanced.glsl"),
    ("ref_first", "res/first_voxelize.glsl"),
    ("ref_second", "res/second_voxelize.glsl"),
    ("ref_cone", "res/conetrace_frag.glsl"),
]
FLAGS = ["-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-w",
         "-fvisibility=hidden"]


def available():
    return all(os.path.exists(os.path.join(REFERENCE, rel)) for _, rel in SHADERS)


def translation_unit():
    parts = ['#include "glsl_shim.hpp"\n']
    for ns, rel in SHADERS:
        path = os.path.join(REFERENCE, rel)
        with open(path) as f:
            lines = f.read().split("\n")
        lines = ["" if ln.lstrip().startswith("#version") else ln for ln in lines]
        # `inout T name` parameters become C++ references (GLSL copies them back)
        lines = [re.sub(r"\binout\s+(\w+)\s+(\w+)", r"\1& \2", ln) for ln in lines]
        parts.append(f"namespace {ns} {{\nusing namespace glsl;\n"
                     "vec4 gl_Position; vec4 gl_FragCoord; float gl_FragDepth;\n"
                     f'#line 1 "{rel}"\n')
        parts.append("\n".join(lines))
        parts.append(f"\n}}  // namespace {ns}\n")
    parts.append('#include "glsl_shim_end.hpp"\n#include "ref_driver.inc"\n')
    return "".join(parts)


def build(force=False):
    """Build the library when the reference is present; returns its path or None."""
    if not available():
        return None
    deps = [os.path.abspath(__file__)] + [os.path.join(SHIM, f) for f in os.listdir(SHIM)]
    deps += [os.path.join(REFERENCE, rel) for _, rel in SHADERS]
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(
            os.path.getmtime(d) for d in deps):
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    cxx = os.environ.get("CXX", "g++")
    cmd = [cxx] + FLAGS + ["-I", SHIM, "-x", "c++", "-", "-o", LIB]
    r = subprocess.run(cmd, input=translation_unit(), capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference shader build failed:\n" + " ".join(cmd) + "\n" + r.stderr)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
