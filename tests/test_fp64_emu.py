"""The integer emulation of binary64 add/sub/mul (csrc/fp64_emu.cuh) against
IEEE-754 hardware arithmetic, on the host (the same source the FP64 step
kernels compile; the GPU parity tests check it in the kernels)."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "imexlb-1.0_gb300", "csrc")
SRC = os.path.join(ROOT, "tests", "fp64_emu_check.cpp")
N = 3_000_000


def _run(tmp_path, extra):
    exe = str(tmp_path / ("emu" + "".join(extra).replace("-", "_")))
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", CSRC, *extra,
                           "-o", exe, SRC])
    out = subprocess.check_output([exe, str(N)], text=True)
    last = out.strip().splitlines()[-1].split()
    assert last[0] == "pairs_per_kind"
    return out, int(last[1]), [int(x) for x in last[3:9]]


def test_emulation_is_bit_exact(tmp_path):
    out, per, bad = _run(tmp_path, [])
    assert sum(bad) == 0, out


def test_emulation_computes_the_common_cases_itself(tmp_path):
    """The hand-off to the hardware instruction is for specials only: on
    normal operands with normal results (distributions 1 and 3) the
    emulation answers every pair itself; where exact cancellation occurs (2,
    and rarely 5) it hands off only the exact zeros."""
    out, per, other = _run(tmp_path, ["-DCOUNT_OTHER"])
    ops = 3 * per
    assert other[1] == 0 and other[3] == 0, out
    assert other[5] < 1e-4 * ops, out
    assert other[2] < 0.05 * ops, out
    assert other[4] > 0.2 * ops, out  # the specials really are handed off
