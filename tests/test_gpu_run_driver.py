"""The imexlb_run driver (main.f90's structure on the GPU) against the oracle.

imexlb_run reads input.in, sets up on the host, advances one Monitor interval
per imexlb_step call, prints `T=` and `Umax=` as Monitor does
(lbm.f90:222-226) and writes output_<count>.plt (main.f90:73). Its Monitor
lines must be the oracle's values scaled and formatted the same way, so the
text matches character for character, and its PLT file must hold the same
records as the file the same writer makes from the oracle's final p and u
(header bytes equal, values equal as IEEE numbers: the sign of an exact zero
may differ).
"""
import os
import subprocess

import numpy as np
import pytest

from parity_util import assert_same
from test_plt import _parse

pytestmark = pytest.mark.gpu

EXE = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                   "imexlb-1.0_gb300", "_build", "imexlb_run")

# input.in / input_3d.in: lattice; L, Xpos, Re; ome, dt, rho0; max_t, inter
INPUTS = {2: "64 32\n0.125 0.25 20\n1.8 1 1\n0.5 0.01\n",
          3: "32 16 16\n0.25 0.25 20\n1.7 1 0.9\n0.5 0.01\n"}


def _same_plt(a, b, dim):
    head, nv = _parse(a, dim)
    start = head["data_offset"] - 8 * 2 * nv  # the min/max limits, then the data
    assert len(a) == len(b) and (len(a) - start) % 8 == 0
    assert a[:start] == b[:start], "PLT header records differ"
    assert_same(np.frombuffer(a, "<f8", offset=start), np.frombuffer(b, "<f8", offset=start),
                "PLT limits and data")


@pytest.mark.parametrize("dim", [2, 3])
def test_driver_matches_oracle(built, tmp_path, dim):
    import imexlb as im
    from oracle import orc
    path = tmp_path / "input.in"
    path.write_text(INPUTS[dim])
    steps, interv, seed = 40, 7, 777
    run = subprocess.run([EXE, str(path), "--dim", str(dim), "--steps", str(steps),
                          "--interv", str(interv), "--seed", str(seed)],
                         cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, run.stderr

    cfg = im.read_input(str(path), dim)
    o = orc.Oracle(orc.read_input(str(path), dim))
    try:
        o.init_up(im.r_vec(seed))
        o.init_pdf()
        log = o.run(0, steps, interv)
        expect = []
        for k, it in enumerate(range(0, steps, interv)):
            expect.append(" T= %.15g" % (it / cfg.t_intv))
            expect.append(" Umax= %.15g" % (log[k] / (cfg.charlength * cfg.t_intv)))
        got = [ln for ln in run.stdout.splitlines() if ln.startswith((" T=", " Umax="))]
        assert got == expect

        count = len(log)
        out = tmp_path / ("output_%03d.plt" % count)
        assert out.exists(), os.listdir(tmp_path)
        ref = tmp_path / "oracle.plt"
        im.write_plt(cfg, str(ref), count, steps, o.p, o.u, o.lists["fluid_id"])
        _same_plt(out.read_bytes(), ref.read_bytes(), dim)
    finally:
        o.close()
