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
# the same source with a*b+c contracted into fused multiply-adds where the
# target has them (aarch64: the default of gfortran and nvfortran there), to
# measure how far a reference build that contracts lies from the one that
# does not
LIB_FMA = os.path.join(BUILD, "liborc_fma.so")
SRC = [os.path.join(HERE, "lbm_oracle.c")]
HDR = [os.path.join(HERE, "lbm_oracle.h")]


def _stale(lib):
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    return any(os.path.getmtime(p) > t for p in SRC + HDR + [__file__])


def build(force=False, contract=False):
    """Compile the oracle shared library (contract: the fused multiply-add
    build) if it is missing or stale; return its path."""
    os.makedirs(BUILD, exist_ok=True)
    lib = LIB_FMA if contract else LIB
    if not force and not _stale(lib):
        return lib
    tmp = lib + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O3", "-std=c11", "-ffp-contract=fast" if contract else "-ffp-contract=off",
           "-fno-fast-math", "-fPIC", "-shared", "-fopenmp", "-o", tmp] + SRC + ["-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, contract="--contract" in sys.argv))
