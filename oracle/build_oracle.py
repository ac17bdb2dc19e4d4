"""Builds the CPU oracle (test infrastructure) as oracle/liboracle.so.

gcc -O2 with -ffp-contract=off and no fast-math: the oracle's FP32 ray
set-up must round operation by operation like the CUDA kernels' explicit
round-to-nearest intrinsics.

The reference's own code for this path cannot be compiled here: the
renderer is an un-vendored external project and the frame glue needs
libswscale/libavcodec/libprotobuf, none of which is installed.  So nothing is
built into oracle/_ref.

    python oracle/build_oracle.py
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "nes_oracle.c")
LIB = os.path.join(HERE, "liboracle.so")
FLAGS = ["-O2", "-fPIC", "-shared", "-std=c11", "-ffp-contract=off", "-fno-fast-math",
         "-pthread"]


def build(force=False):
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    tmp = LIB + ".tmp"
    cmd = [os.environ.get("CC", "gcc")] + FLAGS + [SRC, "-o", tmp, "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed\n" + r.stdout + r.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
