"""Divergence watchdog of imexlb_step (imexlb_set_watchdog).

The reference's Monitor (lbm.f90:205-227) prints whatever maximum it finds,
NaN included, and the run carries on; the library does the same unless the
watchdog is on, in which case the step call fails with IMEXLB_ERR_DIVERGED.
The diverged state is made on the host: one fluid node's uploaded velocity
is NaN (or infinite), which the first Monitor of the call sees. No kernel is
made to fault.
"""
import numpy as np
import pytest

from parity_util import make_case

pytestmark = pytest.mark.gpu


def _case(bad):
    cfg, st, o = make_case("3d_32x16x16")
    u = o.u.copy()
    node = int(st.fluid_id[len(st.fluid_id) // 2])  # not fluid_id(0)
    u[node * cfg.dim] = bad
    return cfg, st, o, u


@pytest.mark.parametrize("bad", [np.nan, np.inf])
def test_watchdog_flags_a_non_finite_monitor(built, bad):
    import imexlb as im
    cfg, st, o, u = _case(bad)
    with im.Solver(cfg) as s:
        s.set_geometry(st)
        s.upload(o.f, o.fb, o.p, u)
        s.set_watchdog(True)
        with pytest.raises(im.ImexlbError) as ei:
            s.step(0, 3, 1)
        assert ei.value.code == im.ERR_DIVERGED
        assert "iteration 0" in str(ei.value)


def test_watchdog_off_keeps_the_reference_behaviour(built):
    import imexlb as im
    cfg, st, o, u = _case(np.nan)
    with im.Solver(cfg) as s:
        s.set_geometry(st)
        s.upload(o.f, o.fb, o.p, u)
        log = s.step(0, 3, 1)
        assert np.isnan(log[0])


def test_watchdog_on_a_healthy_run(built):
    import imexlb as im
    cfg, st, o = make_case("3d_32x16x16")
    with im.Solver(cfg) as s:
        s.set_geometry(st)
        s.upload(o.f, o.fb, o.p, o.u)
        s.set_watchdog(True)
        log = s.step(0, 20, 4)
        assert np.all(np.isfinite(log))
        # the watchdog reads the Monitor values even when the caller does not
        assert im.lib().imexlb_step(s.h, 20, 8, 4, None) == im.IMEXLB_OK
