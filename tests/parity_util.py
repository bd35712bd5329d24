"""Shared helpers for parity tests: build one case on the oracle and the library."""
import numpy as np


def same(a, b):
    """IEEE equality elementwise, NaN matching NaN (bit-exact up to the sign of zero)."""
    a = np.asarray(a)
    b = np.asarray(b)
    return (a == b) | (np.isnan(a) & np.isnan(b))


def assert_same(a, b, what):
    ok = same(a, b)
    if not ok.all():
        bad = np.flatnonzero(~ok)
        i = bad[0]
        raise AssertionError("%s differs at %d of %d slots; first at %d: %r vs %r"
                             % (what, bad.size, ok.size, i, a[i], b[i]))


CASES = {
    # name: (dim, nx, ny, nz, input.in line 2 (L, Xpos, Re), line 3 (ome, dt, rho0))
    "2d_64x32": (2, 64, 32, 0, (0.125, 0.25, 20.0), (1.8, 1.0, 1.0)),
    "2d_48x20_rho": (2, 48, 20, 0, (0.2, 0.3, 30.0), (1.6, 1.0, 1.25)),
    "3d_32x16x16": (3, 32, 16, 16, (0.25, 0.25, 20.0), (1.8, 1.0, 1.0)),
    "3d_24x12x14_rho": (3, 24, 12, 14, (0.3, 0.35, 15.0), (1.7, 1.0, 0.9)),
}


def make_case(name, seed=12345):
    """(cfg, setup) from the library's host setup, and the matching oracle."""
    import imexlb as im
    from oracle import orc
    dim, nx, ny, nz, (L, xp, re), (ome, dt, rho0) = CASES[name]
    cfg = im.make_config(dim, nx, ny, nz, charlength=L, xpos=xp, re=re, ome=ome, dt=dt, rho0=rho0)
    st = im.Setup(cfg, seed=seed)
    o = orc.Oracle(orc.make_input(dim, nx, ny, nz, charlength=L, xpos=xp, re=re, ome=ome, dt=dt,
                                  rho0=rho0))
    o.init_up(st.r_vec)
    o.init_pdf()
    return cfg, st, o
