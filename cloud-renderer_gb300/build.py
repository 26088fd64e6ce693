"""Build recipe for libcloudgb.so (sm_103a) and the CPU oracle.

Everything is compiled in-tree with nvcc/gcc directly (no cmake): one
translation unit per file, compiled in parallel, linked into
cloud-renderer_gb300/cloudgb/libcloudgb.so.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT_DIR = os.path.join(PKG, "cloudgb")
# CG_BOUNDS_CHECK=1: the bounds-check build (csrc/cg_check.cuh), a separate
# library with its own objects
CHECK = os.environ.get("CG_BOUNDS_CHECK") == "1"
BUILD_DIR = os.path.join(PKG, "_build_check" if CHECK else "_build")
LIB = os.path.join(OUT_DIR, "libcloudgb_check.so" if CHECK else "libcloudgb.so")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# (source, extra flags).  The voxelization kernels decide indices with FP32
# arithmetic that must match the oracle bit for bit: no FMA contraction.
SOURCES = [
    ("cg_host.cpp", ["-Xcompiler", "-ffp-contract=off"]),
    ("k_voxelize.cu", ["-fmad=false"]),
    ("k_trace.cu", []),
    ("k_noalloc.cu", []),
    ("k_deferred.cu", []),
    ("k_mlp.cu", []),
    ("k_textures.cu", []),
    ("k_shade_tc.cu", []),
    ("k_render_tc.cu", []),
    ("k_train_tc.cu", []),
    ("k_stats.cu", []),
    ("k_batch.cu", []),
    ("cg_batch.cpp", ["-Xcompiler", "-ffp-contract=off"]),
    ("cg_mlp.cpp", ["-Xcompiler", "-ffp-contract=off"]),
    ("k_compat.cu", []),
    ("cg_compat.cpp", ["-Xcompiler", "-ffp-contract=off"]),
]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _newer(target, deps):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def build_library(force=False, verbose=False):
    os.makedirs(BUILD_DIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "cloudgb.h"))
    common = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
              "-I", CSRC, "-I", os.path.join(ROOT, "include")] + ARCH
    if CHECK:
        common.append("-DCG_BOUNDS_CHECK=1")
    objs, jobs = [], []
    for src, extra in SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(BUILD_DIR, src + ".o")
        objs.append(obj)
        if force or not _newer(obj, [path] + headers + [os.path.abspath(__file__)]):
            jobs.append([NVCC, "-c", path, "-o", obj] + common + extra)
    if jobs:
        with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            for out in ex.map(_run, jobs):
                if verbose and out.strip():
                    print(out)
    if force or jobs or not os.path.exists(LIB):
        _run([NVCC, "-shared", "-o", LIB] + objs + ARCH + ["-lcudart_static", "-lrt", "-lpthread", "-ldl"])
    return LIB


if __name__ == "__main__":
    print(build_library(force="--force" in sys.argv, verbose=True))
