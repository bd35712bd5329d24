"""GPU parity: libimexlb's FP64 path against the CPU oracle, bit for bit.

Every comparison is IEEE equality (NaN matches NaN): the kernels round every
operation as the reference's serial build does, so the only admissible
difference is the sign of an exact zero.
"""
import numpy as np
import pytest

from parity_util import CASES, assert_same, make_case

pytestmark = pytest.mark.gpu


def _solver(cfg, st, o):
    import imexlb as im
    s = im.Solver(cfg)
    s.set_geometry(st)
    # the oracle holds InitUP + InitPDF; fb is all zero as allocated
    s.upload(o.f, o.fb, o.p, o.u)
    return s


@pytest.mark.parametrize("name", sorted(CASES))
def test_steps_match_oracle(built, name):
    cfg, st, o = make_case(name)
    with _solver(cfg, st, o) as s:
        interv = 7
        log_g = s.step(0, 40, interv)
        log_o = o.run(0, 40, interv)
        assert_same(log_g, log_o, "Monitor")
        f, fb, p, u = s.download()
        assert_same(f, o.f, "f")
        assert_same(p, o.p, "p")
        assert_same(u, o.u, "u")
        assert_same(fb, o.fb, "fb")


def test_init_pdf_on_device(built):
    cfg, st, o = make_case("3d_32x16x16")
    import imexlb as im
    with im.Solver(cfg) as s:
        s.set_geometry(st)
        s.upload(np.zeros_like(o.f), o.fb, o.p, o.u)
        s.init_pdf()
        f, _, _, _ = s.download()
        assert_same(f, o.f, "InitPDF f")


def test_chunked_steps_and_midrun_download(built):
    cfg, st, o = make_case("2d_64x32")
    with _solver(cfg, st, o) as s:
        logs = []
        for it0, n in ((0, 5), (5, 1), (6, 17), (23, 2)):
            logs.append(s.step(it0, n, 4))
            s.download()  # reading the state must not disturb it
        log_g = np.concatenate(logs)
        log_o = o.run(0, 25, 4)
        assert_same(log_g, log_o, "Monitor")
        f, fb, p, u = s.download()
        assert_same(f, o.f, "f")
        assert_same(fb, o.fb, "fb")
        assert_same(p, o.p, "p")
        assert_same(u, o.u, "u")


def test_reupload_restarts_from_host_state(built):
    cfg, st, o = make_case("3d_24x12x14_rho")
    with _solver(cfg, st, o) as s:
        s.step(0, 9, 0)
        o.run(0, 9, 0)
        f, fb, p, u = s.download()
        # continue on the oracle; restart the device from the downloaded state
        s.upload(f, fb, p, u)
        log_g = s.step(9, 11, 5)
        log_o = o.run(9, 11, 5)
        assert_same(log_g, log_o, "Monitor")
        f, fb, p, u = s.download()
        assert_same(f, o.f, "f")
        assert_same(fb, o.fb, "fb")


def test_zero_steps_is_identity(built):
    cfg, st, o = make_case("2d_48x20_rho")
    with _solver(cfg, st, o) as s:
        assert s.step(0, 0, 1).size == 0
        f, fb, p, u = s.download()
        assert_same(f, o.f, "f")
        assert_same(p, o.p, "p")
        assert_same(u, o.u, "u")


@pytest.mark.parametrize("name", ["2d_64x32", "3d_32x16x16"])
def test_every_fp64_split_matches_oracle(built, name):
    """Each step-kernel variant (a share of the FP64 operations in integer
    emulation) reproduces the oracle bit for bit."""
    import imexlb as im
    cfg, st, o = make_case(name)
    init = [x.copy() for x in (o.f, o.fb, o.p, o.u)]
    log_o = o.run(0, 40, 7)
    for v in range(im.fp64_splits()):
        with im.Solver(cfg) as s:
            s.set_geometry(st)
            s.upload(*init)
            s.set_fp64_split(v)
            log_g = s.step(0, 40, 7)
            assert_same(log_g, log_o, "Monitor (split %d)" % v)
            f, fb, p, u = s.download()
            assert_same(f, o.f, "f (split %d)" % v)
            assert_same(fb, o.fb, "fb (split %d)" % v)
            assert_same(p, o.p, "p (split %d)" % v)
            assert_same(u, o.u, "u (split %d)" % v)


def test_fp64_split_range_is_checked(built):
    import imexlb as im
    cfg, st, o = make_case("2d_64x32")
    with im.Solver(cfg) as s:
        with pytest.raises(im.ImexlbError):
            s.set_fp64_split(im.fp64_splits())
        with pytest.raises(im.ImexlbError):
            s.set_fp64_split(-1)


@pytest.mark.parametrize("name", ["2d_64x32", "3d_32x16x16"])
def test_corrected_physics_matches_oracle(built, name):
    """The corrected-physics obstacle list (every solid link bounced) through
    the library against the oracle running the same list: bit for bit."""
    import imexlb as im
    from oracle import orc
    from parity_util import CASES
    dim, nx, ny, nz, (L, xp, re), (ome, dt, rho0) = CASES[name]
    cfg = im.make_config(dim, nx, ny, nz, charlength=L, xpos=xp, re=re, ome=ome, dt=dt, rho0=rho0)
    st = im.Setup(cfg, physics="corrected")
    o = orc.Oracle(orc.make_input(dim, nx, ny, nz, charlength=L, xpos=xp, re=re, ome=ome, dt=dt,
                                  rho0=rho0), allow_geom_error=True)
    o.use_corrected_obstacles()
    assert np.array_equal(o.lists["b_user"], st.b_user)
    o.init_up(st.r_vec)
    o.init_pdf()
    with _solver(cfg, st, o) as s:
        log_g = s.step(0, 40, 7)
        log_o = o.run(0, 40, 7)
        assert_same(log_g, log_o, "Monitor")
        f, fb, p, u = s.download()
        assert_same(f, o.f, "f")
        assert_same(fb, o.fb, "fb")
        assert_same(p, o.p, "p")
        assert_same(u, o.u, "u")


@pytest.mark.parametrize("name", ["2d_64x32", "3d_32x16x16", "2d_48x20_rho"])
@pytest.mark.parametrize("rest", [False, True])
def test_device_initial_state_equals_host_upload(built, name, rest):
    """imexlb_init_state (InitUP on the device, or the rest state) gives the
    same bits as the host's InitUP uploaded with zero f and fb."""
    import imexlb as im
    cfg, st, o = make_case(name)
    p, u = st.p.copy(), st.u.copy()
    if rest:
        p[:] = 0.0
        u[:] = 0.0
    with im.Solver(cfg) as a, im.Solver(cfg) as b:
        for s in (a, b):
            s.set_geometry(st)
        a.upload(np.zeros_like(st.f), np.zeros_like(st.fb), p, u)
        b.init_state(None if rest else st.r_vec)
        for s in (a, b):
            s.init_pdf()
        ra, rb = a.download(), b.download()
        for x, y, what in zip(ra, rb, ("f", "fb", "p", "u")):
            assert np.array_equal(x.view(np.uint64), y.view(np.uint64)), what
        la, lb = a.step(0, 12, 5), b.step(0, 12, 5)
        assert_same(la, lb, "Monitor")
