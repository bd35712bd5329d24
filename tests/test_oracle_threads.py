"""The oracle's results do not depend on its OpenMP thread count.

The full-size GPU parity tests and the CPU reference arm run the oracle over
all host cores; the bitwise comparisons elsewhere use one thread. Its
parallel loops are per cell (Collision, Propagation, PostProcessing) and the
Monitor maximum does not depend on order, so every bit must agree.
"""
import os

import numpy as np
import pytest

from oracle import orc


def _run(nthreads, dim, n, kw, steps, interv):
    o = orc.Oracle(orc.make_input(dim, *n, **kw), nthreads=nthreads)
    try:
        o.init_up(orc.r_vec(99))
        o.init_pdf()
        log = o.run(0, steps, interv)
        return [a.copy() for a in (o.f, o.fb, o.p, o.u)], log
    finally:
        o.close()


@pytest.mark.parametrize("dim,n", [(2, (96, 40, 0)), (3, (40, 20, 24))])
def test_thread_count_does_not_change_bits(built, dim, n):
    kw = dict(charlength=0.2, xpos=0.3, re=40.0, ome=1.8, dt=1.0, rho0=1.0)
    many = max(4, os.cpu_count() or 1)
    one, log1 = _run(1, dim, n, kw, 25, 4)
    par, logp = _run(many, dim, n, kw, 25, 4)
    assert np.array_equal(log1.view(np.uint64), logp.view(np.uint64))
    for a, b, name in zip(one, par, ("f", "fb", "p", "u")):
        assert np.array_equal(a.view(np.uint64), b.view(np.uint64)), name
