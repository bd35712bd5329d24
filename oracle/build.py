"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/lbm_oracle.c into oracle/_build/liborc.so with gcc:
-O3 with -ffp-contract=off and no fast-math keeps every a*b+c unfused and
every sum in source order, so the oracle rounds like the reference's serial
build; -fopenmp parallelises only the per-cell loops, whose results do not
depend on the thread count.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liborc.so")
SRC = [os.path.join(HERE, "lbm_oracle.c")]
HDR = [os.path.join(HERE, "lbm_oracle.h")]


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(p) > t for p in SRC + HDR + [__file__])


def build(force=False):
    """Compile the oracle shared library if it is missing or stale; return its path."""
    os.makedirs(BUILD, exist_ok=True)
    if not force and not _stale():
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O3", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fPIC",
           "-shared", "-fopenmp", "-o", tmp] + SRC + ["-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
