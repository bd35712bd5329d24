"""Boundary copies inside the step kernel (IMEXLB_FILL_FUSED) against the
separate fill kernel (IMEXLB_FILL_KERNEL) and the oracle.

The reference's BoundaryCondition (lbm.f90:96-155, lbm_3d.f90:96-157)
resolves to slot-to-slot copies that no other copy reads. In fused mode a
node that pulls a ghost slot reads the copy's source (closed forms on the
inlet and outlet columns, a source row elsewhere) and obstacle slots are
written by the thread that wrote their source. FP64 stays bit-exact with the
oracle and every storage kind gives the same bits in both modes."""
import numpy as np
import pytest

from parity_util import CASES, assert_same, make_case

pytestmark = pytest.mark.gpu


def _run(cfg, st, init, mode, steps, interv, precision=0, chunks=(None,), observe=False):
    import imexlb as im
    with im.Solver(cfg, precision=precision) as s:
        s.set_geometry(st)
        s.upload(*init)
        log, obs = [], []
        it = 0
        for k, m in enumerate(chunks):
            s.set_fill_mode(mode if m is None else m)
            n = steps // len(chunks) if k < len(chunks) - 1 else steps - it
            log.append(s.step(it, n, interv))
            if observe:
                obs.append(s.observe())
            it += n
        return np.concatenate(log), s.download(), s.fill_mode(), obs


@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("mode", ["kernel", "fused"])
def test_both_modes_match_oracle(built, name, mode):
    import imexlb as im
    m = im.FILL_FUSED if mode == "fused" else im.FILL_KERNEL
    cfg, st, o = make_case(name)
    init = [x.copy() for x in (o.f, o.fb, o.p, o.u)]
    log_o = o.run(0, 30, 6)
    log_g, (f, fb, p, u), used, _ = _run(cfg, st, init, m, 30, 6)
    assert used == m
    assert_same(log_g, log_o, "Monitor")
    for a, b, w in ((f, o.f, "f"), (fb, o.fb, "fb"), (p, o.p, "p"), (u, o.u, "u")):
        assert_same(a, b, w)


@pytest.mark.parametrize("name", ["2d_64x32", "3d_32x16x16"])
def test_corrected_physics_in_fused_mode(built, name):
    """More obstacle copies (every wetted solid cell): the pushed copies."""
    import imexlb as im
    from oracle import orc
    dim, nx, ny, nz, (L, xp, re), (ome, dt, rho0) = CASES[name]
    cfg = im.make_config(dim, nx, ny, nz, charlength=L, xpos=xp, re=re, ome=ome, dt=dt, rho0=rho0)
    st = im.Setup(cfg, seed=3, physics="corrected")
    o = orc.Oracle(orc.make_input(dim, nx, ny, nz, charlength=L, xpos=xp, re=re, ome=ome, dt=dt,
                                  rho0=rho0), allow_geom_error=True)
    o.use_corrected_obstacles()
    o.init_up(st.r_vec)
    o.init_pdf()
    init = [x.copy() for x in (o.f, o.fb, o.p, o.u)]
    log_o = o.run(0, 25, 5)
    log_g, (f, fb, p, u), used, _ = _run(cfg, st, init, im.FILL_FUSED, 25, 5)
    assert used == im.FILL_FUSED
    assert_same(log_g, log_o, "Monitor")
    for a, b, w in ((f, o.f, "f"), (fb, o.fb, "fb"), (p, o.p, "p"), (u, o.u, "u")):
        assert_same(a, b, w)


def test_switching_modes_between_calls(built):
    """Mode changes between imexlb_step calls (the captured two-iteration
    graph is rebuilt, the ghost slots brought up to date) keep the run on the
    oracle's bits; observe() in between reads the same mass and force."""
    import imexlb as im
    cfg, st, o = make_case("3d_24x12x14_rho")
    init = [x.copy() for x in (o.f, o.fb, o.p, o.u)]
    o.run(0, 41, 0)
    chunks = (im.FILL_FUSED, im.FILL_KERNEL, im.FILL_FUSED, im.FILL_KERNEL, im.FILL_FUSED)
    _, (f, fb, p, u), _, obs_a = _run(cfg, st, init, None, 41, 0, chunks=chunks, observe=True)
    for a, b, w in ((f, o.f, "f"), (fb, o.fb, "fb"), (p, o.p, "p"), (u, o.u, "u")):
        assert_same(a, b, w)
    _, _, _, obs_b = _run(cfg, st, init, im.FILL_KERNEL, 41, 0, chunks=(None,) * 5, observe=True)
    for (Fa, ma), (Fb, mb) in zip(obs_a, obs_b):
        assert np.array_equal(Fa, Fb) and ma == mb


@pytest.mark.parametrize("name", ["2d_64x32", "3d_32x16x16"])
@pytest.mark.parametrize("prec", ["fp64fast", "fp32", "bf16", "fp16", "fix64"])
def test_modes_agree_bitwise_in_every_storage_kind(built, name, prec):
    import imexlb as im
    code = {"fp64fast": im.FP64_FAST, "fp32": im.FP32, "bf16": im.BF16, "fp16": im.FP16,
            "fix64": im.FIX64}[prec]
    cfg, st, o = make_case(name)
    init = [x.copy() for x in (o.f, o.fb, o.p, o.u)]
    a = _run(cfg, st, init, im.FILL_KERNEL, 35, 5, precision=code, observe=True)
    b = _run(cfg, st, init, im.FILL_FUSED, 35, 5, precision=code, observe=True)
    assert b[2] == im.FILL_FUSED
    assert np.array_equal(a[0].view(np.uint64), b[0].view(np.uint64))
    for x, y, w in zip(a[1], b[1], ("f", "fb", "p", "u")):
        assert np.array_equal(np.asarray(x).view(np.uint64), np.asarray(y).view(np.uint64)), w
    assert np.array_equal(a[3][0][0], b[3][0][0]) and a[3][0][1] == b[3][0][1]


def test_sample_after_fused_steps(built):
    import imexlb as im
    cfg, st, o = make_case("2d_64x32")
    init = [x.copy() for x in (o.f, o.fb, o.p, o.u)]
    out = []
    for mode in (im.FILL_KERNEL, im.FILL_FUSED):
        with im.Solver(cfg, precision=im.FP32) as s:
            s.set_geometry(st)
            s.upload(*init)
            s.set_fill_mode(mode)
            s.step(0, 20, 0)
            out.append(s.sample(96, 48))
    assert np.array_equal(out[0], out[1])


def test_obstacle_next_to_a_wall_keeps_the_separate_kernel(built):
    """An obstacle cell one row inside the wall: the wall's ghost copy reads
    its slot before the obstacle copies rewrite it (a value of the previous
    iteration), which no pull of the next step can read. Fused mode is
    refused and the results stay the oracle-checked ones of the separate
    kernel."""
    import imexlb as im
    cfg, st, o = make_case("2d_64x32")
    geo = st.geo.copy()
    lists = {k: getattr(st, k).copy() for k in ("fluid_id", "bl", "br", "bu", "bd", "b_user")}
    cell = (20 + 3) + cfg.dy * (1 + 3)  # x = 20, y = 1
    assert geo[cell] == 1
    geo[cell] = 0
    lists["fluid_id"] = lists["fluid_id"][lists["fluid_id"] != cell]
    lists["b_user"] = np.sort(np.append(lists["b_user"], cell))
    with im.Solver(cfg) as s:
        s.set_geometry(geo=geo, **lists)
        assert s.fill_mode() == im.FILL_KERNEL
        with pytest.raises(im.ImexlbError) as e:
            s.set_fill_mode(im.FILL_FUSED)
        assert e.value.code == im.ERR_UNSUPPORTED
        s.set_fill_mode(im.FILL_KERNEL)


def test_fill_mode_argument_is_checked(built):
    import imexlb as im
    cfg, st, o = make_case("2d_64x32")
    with im.Solver(cfg) as s:
        assert s.fill_mode() == im.FILL_KERNEL  # no geometry yet: nothing to fuse
        with pytest.raises(im.ImexlbError):
            s.set_fill_mode(7)
        s.set_geometry(st)
        assert s.fill_mode() == im.FILL_FUSED
        s.set_fill_mode(im.FILL_KERNEL)
        assert s.fill_mode() == im.FILL_KERNEL


@pytest.mark.parametrize("name,prec,mode", [("3d_32x16x16", "fp64", "fused"),
                                            ("3d_32x16x16", "fp16", "fused"),
                                            ("2d_64x32", "fp64", "fused"),
                                            ("2d_64x32", "fp32", "fused")])
def test_default_mode(built, name, prec, mode):
    import imexlb as im
    code = {"fp64": im.FP64, "fp16": im.FP16, "fp32": im.FP32}[prec]
    cfg, st, o = make_case(name)
    with im.Solver(cfg, precision=code) as s:
        s.set_geometry(st)
        assert s.fill_mode() == (im.FILL_FUSED if mode == "fused" else im.FILL_KERNEL)


def test_fp64_variants_other_than_the_default_use_the_separate_kernel(built):
    import imexlb as im
    cfg, st, o = make_case("2d_64x32")
    init = [x.copy() for x in (o.f, o.fb, o.p, o.u)]
    log_o = o.run(0, 20, 5)
    with im.Solver(cfg) as s:
        s.set_geometry(st)
        s.upload(*init)
        assert s.fill_mode() == im.FILL_FUSED
        s.set_fp64_split(0)
        assert s.fill_mode() == im.FILL_KERNEL
        log_g = s.step(0, 20, 5)
        assert_same(log_g, log_o, "Monitor")
        f, fb, p, u = s.download()
        assert_same(fb, o.fb, "fb")


def test_batch_after_fused_steps(built):
    """A batch runs each case's fill list after every step; cases whose own
    fused steps left the ghost slots out get them written first."""
    import imexlb as im
    cfg, st, o = make_case("2d_64x32")
    out = []
    for batched in (False, True):
        s = im.Solver(cfg, precision=im.FP32)
        s.set_geometry(st)
        s.upload(st.f, st.fb, st.p, st.u)
        s.init_pdf()
        assert s.fill_mode() == im.FILL_FUSED
        s.step(0, 11)
        if batched:
            with im.Batch([s]) as b:
                b.step(nsteps=20)
        else:
            s.step(11, 20)
        out.append(s.download())
        s.close()
    for a, b2, w in zip(out[0], out[1], ("f", "fb", "p", "u")):
        fin = np.isfinite(a)
        assert np.array_equal(fin, np.isfinite(b2)), w
        scale = np.abs(a[fin]).max()
        # the batched kernel may contract multiply-adds differently
        assert np.abs(a[fin] - b2[fin]).max() <= 2e-6 * scale, w


@pytest.mark.parametrize("dim,n,steps,prec", [(2, (256, 128, 0), 2000, "fp64"), (3, (64, 32, 32), 300, "fp64"),
                                              (2, (256, 128, 0), 2000, "fp16"), (3, (64, 32, 32), 300, "fp16")])
def test_modes_agree_over_long_runs(built, dim, n, steps, prec):
    """Both boundary-copy modes over many iterations of a flow past the
    obstacle: the same bits, and the same Monitor log and force."""
    import imexlb as im
    code = {"fp64": im.FP64, "fp16": im.FP16}[prec]
    cfg = im.make_config(dim, *n, charlength=0.125 if dim == 2 else 0.25, xpos=0.25, re=80.0,
                         ome=1.7)
    st = im.Setup(cfg, seed=21)
    res = []
    for mode in (im.FILL_KERNEL, im.FILL_FUSED):
        with im.Solver(cfg, precision=code) as s:
            s.set_geometry(st)
            s.set_fill_mode(mode)
            s.upload(st.f, st.fb, st.p, st.u)
            s.init_pdf()
            log = s.step(0, steps, 97)
            F, mass = s.observe()
            res.append((log, F, mass) + tuple(s.download()))
    a, b = res
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]) and a[2] == b[2]
    for x, y in zip(a[3:], b[3:]):
        assert np.array_equal(np.asarray(x).view(np.uint64), np.asarray(y).view(np.uint64))


def _agree(cfg, geo, lists, init, steps, interv, precision=0):
    import imexlb as im
    out = []
    for mode in (im.FILL_KERNEL, im.FILL_FUSED):
        with im.Solver(cfg, precision=precision) as s:
            s.set_geometry(geo=geo, **lists)
            s.set_fill_mode(mode)
            assert s.fill_mode() == mode
            s.upload(*init)
            log = s.step(0, steps, interv)
            out.append((log,) + tuple(s.download()))
    for x, y in zip(out[0], out[1]):
        assert np.array_equal(np.asarray(x).view(np.uint64), np.asarray(y).view(np.uint64))


@pytest.mark.parametrize("dim", [2, 3])
def test_obstacle_touching_the_inlet_in_both_modes(built, dim):
    """Obstacle cells in the first interior columns: the inlet copies read
    obstacle slots the obstacle copies wrote (record nodes at the rim)."""
    import imexlb as im
    n = (40, 24, 0) if dim == 2 else (24, 12, 12)
    cfg = im.make_config(dim, *n, charlength=0.2, xpos=0.5, re=30.0, ome=1.7)
    st = im.Setup(cfg, seed=4)
    geo = st.geo.copy()
    lists = {k: getattr(st, k).copy() for k in ("fluid_id", "bl", "br", "bu", "bd", "b_user")}
    yz = [(y, z) for y in (5, 6, 7) for z in ((0,) if dim == 2 else (5, 6))]
    cells = [(x + 3) + cfg.dy * (y + 3) + (cfg.dz * (z + 3) if dim == 3 else 0)
             for x in (0, 1) for (y, z) in yz]
    for c in cells:
        geo[c] = 0
        lists["fluid_id"] = lists["fluid_id"][lists["fluid_id"] != c]
    lists["b_user"] = np.sort(np.concatenate([lists["b_user"], cells]))
    _agree(cfg, geo, lists, (st.f, st.fb, st.p, st.u), 60, 7)


@pytest.mark.parametrize("n", [(63, 31, 0), (45, 20, 0), (31, 15, 17), (20, 13, 9)])
def test_odd_lattices_in_both_modes(built, n):
    import imexlb as im
    dim = 2 if n[2] == 0 else 3
    cfg = im.make_config(dim, *n, charlength=0.25, xpos=0.3, re=25.0, ome=1.75)
    st = im.Setup(cfg, seed=8)
    lists = {k: getattr(st, k) for k in ("fluid_id", "bl", "br", "bu", "bd", "b_user")}
    for prec in (im.FP64, im.FP16):
        _agree(cfg, st.geo, lists, (st.f, st.fb, st.p, st.u), 50, 9, precision=prec)
