"""GPU: momentum-exchange force and mass against the oracle.

Both sides accumulate in double-double, so the GPU's fixed tree order and the
oracle's sequential order agree to ~1e-30 relative before the final rounding;
the tolerance is 2 ulp of the largest partial magnitude.
"""
import numpy as np
import pytest

from parity_util import make_case

pytestmark = pytest.mark.gpu


def _close(a, b, scale):
    return np.all(np.abs(np.asarray(a) - np.asarray(b)) <= 4.5e-16 * scale)


@pytest.mark.parametrize("name", ["2d_64x32", "3d_32x16x16", "3d_24x12x14_rho"])
def test_observe_matches_oracle(built, name):
    import imexlb as im
    cfg, st, o = make_case(name)
    with im.Solver(cfg) as s:
        s.set_geometry(st)
        s.upload(o.f, o.fb, o.p, o.u)
        # as uploaded: oracle state after InitPDF, fb all zero
        F0, m0 = s.observe()
        Fo, nlinks = o.forces()
        assert s.info().n_links == nlinks > 0
        assert _close(F0, Fo, 1.0) and _close(m0, o.mass(), abs(o.f).sum())
        s.step(0, 17, 0)
        o.run(0, 17, 0)
        F, m = s.observe()
        Fo, _ = o.forces()
        fbv = o.fb.reshape(-1, o.s.nq)
        scale = 2 * np.abs(fbv[o.lists["fluid_id"]]).sum()
        assert _close(F, Fo, scale), (F, Fo)
        assert _close(m, o.mass(), np.abs(o.f).sum()), (m, o.mass())
        assert np.any(F != 0)


def test_force_series_matches_oracle(built):
    import imexlb as im
    cfg, st, o = make_case("2d_48x20_rho")
    every = 3
    with im.Solver(cfg) as s:
        s.set_geometry(st)
        s.upload(o.f, o.fb, o.p, o.u)
        mon, Fs = s.step_observed(0, 20, 5, every)
        ref_F, ref_mon = [], []
        for it in range(20):
            ref_mon.extend(o.run(it, 1, 5).tolist())
            if it % every == 0:
                ref_F.append(o.forces()[0])
        assert np.array_equal(mon, np.array(ref_mon))
        ref_F = np.array(ref_F)
        assert Fs.shape == ref_F.shape
        assert _close(Fs, ref_F, 2 * np.nanmax(np.abs(o.fb)) * o.s.size_fluid * o.s.nq)


def test_fp64_fma_rate_is_plausible(built):
    """The diagnostic DFMA throughput kernel: between 0.05 and 10 T/s (GB300
    issues about 0.6 T FP64 fused multiply-adds per second)."""
    import imexlb as im
    r = im.fp64_fma_rate(0)
    assert 0.05e12 < r < 10e12
