"""Build recipe for the CPU oracle (test infrastructure).

Compiles oracle/cloud_oracle.c twice with gcc:
  liboracle64.so  -- FP64 oracle (the checker)
  liboracle32.so  -- FP32 multithreaded build (the timed CPU baseline)
-ffp-contract=off keeps the FP32 index arithmetic free of FMA contraction on
both x86-64 and aarch64 hosts.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "cloud_oracle.c")
FLAGS = ["-O2", "-std=gnu11", "-fPIC", "-shared", "-pthread", "-ffp-contract=off",
         "-fno-fast-math", "-fvisibility=hidden"]
TARGETS = {
    "liboracle64.so": ["-DOR_REAL=double"],
    "liboracle32.so": ["-DOR_REAL=float", "-DOR_REAL_IS_FLOAT"],
}


def build(force=False):
    cc = os.environ.get("CC", "gcc")
    out = []
    for name, defs in TARGETS.items():
        lib = os.path.join(HERE, name)
        if force or not os.path.exists(lib) or os.path.getmtime(lib) < max(
                os.path.getmtime(SRC), os.path.getmtime(os.path.abspath(__file__))):
            cmd = [cc] + FLAGS + defs + [SRC, "-o", lib, "-lm"]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + r.stderr)
        out.append(lib)
    return out


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
