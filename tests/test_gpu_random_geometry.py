"""GPU parity on random lattices and obstacles.

Seeded draws of the input.in values (lattice size, obstacle size and x
position, relaxation, rho0, and Re through the inlet velocity it gives), the
obstacle rule (the reference's or the corrected one), the Monitor interval
and the way the iterations are split into calls. Each case runs the library
in both boundary-copy modes and the oracle once; f, fb, p, u and the Monitor
values must agree bit for bit (IEEE equality, NaN matching NaN). With FP16,
FP32 and fixed-point storage the two modes must give the same bits. The draws exercise
the in-step boundary plan on geometries nobody chose by hand: obstacles
touching the inlet columns or the walls, thin and odd-sized lattices.
Geometries the reference itself cannot set up (its obstacle probe leaves the
geo array) are refused alike by the host set-up and the oracle and are
skipped; so are geometries whose pulled slots the reference fills from
outside its arrays.
"""
import numpy as np
import pytest

from parity_util import assert_same

pytestmark = pytest.mark.gpu

N_CASES = 14


def _draw(rng, dim):
    return dict(dim=dim, nx=int(rng.integers(20, 97)), ny=int(rng.integers(12, 49)),
                nz=int(rng.integers(12, 41)) if dim == 3 else 0,
                charlength=float(rng.uniform(0.08, 0.35)), xpos=float(rng.uniform(0.15, 0.6)),
                u_in=float(rng.uniform(0.01, 0.1)), ome=float(rng.uniform(1.1, 1.95)),
                rho0=float(rng.uniform(0.8, 1.3)) if rng.random() < 0.4 else 1.0,
                physics="corrected" if rng.random() < 0.3 else "reference",
                interv=int(rng.integers(0, 9)), steps=int(rng.integers(6, 41)),
                seed=int(rng.integers(1, 1 << 30)))


def _chunks(rng, steps):
    """Split `steps` iterations into one to four calls."""
    cuts = sorted(set(int(c) for c in rng.integers(1, steps, size=int(rng.integers(0, 4)))))
    bounds = [0] + cuts + [steps]
    return [(a, b - a) for a, b in zip(bounds, bounds[1:])]


def _cases(dim):
    """(index, draw, call split, config, host set-up, input.in values) of the
    seeded draws whose geometry the host set-up accepts; checks that the
    oracle refuses the others too."""
    import imexlb as im
    from oracle import orc
    rng = np.random.default_rng(20260 + dim)
    for k in range(N_CASES):
        c = _draw(rng, dim)
        chunks = _chunks(rng, c["steps"])
        kw = dict(charlength=c["charlength"], xpos=c["xpos"], re=100.0, ome=c["ome"],
                  rho0=c["rho0"])
        # DataInput derives the inlet velocity in proportion to Re: pick the
        # Re that gives the drawn velocity, so that the flow stays stable
        kw["re"] = 100.0 * c["u_in"] / im.make_config(dim, c["nx"], c["ny"], c["nz"], **kw).uu
        cfg = im.make_config(dim, c["nx"], c["ny"], c["nz"], **kw)
        try:
            st = im.Setup(cfg, seed=c["seed"], physics=c["physics"])
        except im.ImexlbError as e:
            assert e.code == im.ERR_GEOMETRY
            with pytest.raises(ValueError):
                orc.Oracle(orc.make_input(dim, c["nx"], c["ny"], c["nz"], **kw))
            continue
        yield k, c, chunks, cfg, st, kw


def _run(cfg, st, mode, chunks, interv, init, precision=None):
    """Step a fresh handle in `mode` from `init` over the call split; None if
    the device set-up refuses the geometry, else (mode used, Monitor values,
    downloaded state)."""
    import imexlb as im
    with (im.Solver(cfg) if precision is None else im.Solver(cfg, precision=precision)) as s:
        try:
            s.set_geometry(st)
        except im.ImexlbError as e:
            assert e.code == im.ERR_GEOMETRY
            return None
        try:
            s.set_fill_mode(mode)
        except im.ImexlbError as e:
            # no in-step plan for this geometry (an obstacle copy feeding a
            # ghost slot): the separate kernel runs
            assert mode == im.FILL_FUSED and e.code == im.ERR_UNSUPPORTED
        s.upload(*init)
        log = [s.step(it0, n, interv) for it0, n in chunks]
        return s.fill_mode(), np.concatenate(log), s.download()


def _oracle(dim, c, kw, st):
    """The oracle of a draw after InitUP and InitPDF."""
    from oracle import orc
    # the corrected rule does not use the reference's probe, so a probe that
    # leaves geo does not stop it
    o = orc.Oracle(orc.make_input(dim, c["nx"], c["ny"], c["nz"], **kw),
                   allow_geom_error=c["physics"] == "corrected")
    if c["physics"] == "corrected":
        o.use_corrected_obstacles()
    o.init_up(st.r_vec)
    o.init_pdf()
    return o


@pytest.mark.parametrize("dim", [2, 3])
def test_random_geometries_match_oracle(built, dim):
    import imexlb as im
    ran = fused_used = 0
    for k, c, chunks, cfg, st, kw in _cases(dim):
        o = _oracle(dim, c, kw, st)
        try:
            init = (o.f.copy(), o.fb.copy(), o.p.copy(), o.u.copy())
            log_o = o.run(0, c["steps"], c["interv"])
            results = [_run(cfg, st, m, chunks, c["interv"], init)
                       for m in (im.FILL_FUSED, im.FILL_KERNEL)]
            if results[0] is None:
                continue
            ran += 1
            for mode, (used, log_g, (f, fb, p, u)) in zip((im.FILL_FUSED, im.FILL_KERNEL), results):
                what = "case %d %s mode %d" % (k, c, mode)
                fused_used += used == im.FILL_FUSED
                assert_same(log_g, log_o, "Monitor, " + what)
                assert_same(f, o.f, "f, " + what)
                assert_same(fb, o.fb, "fb, " + what)
                assert_same(p, o.p, "p, " + what)
                assert_same(u, o.u, "u, " + what)
        finally:
            o.close()
    # most draws are valid reference geometries, and most of those take the
    # in-step boundary plan
    assert ran >= N_CASES // 2
    assert fused_used >= ran // 2


@pytest.mark.parametrize("dim", [2, 3])
def test_random_geometries_fill_modes_agree_narrow(built, dim):
    """FP16, FP32 and fixed-point storage (the last where rho0 = 1): both
    boundary-copy modes give the same bits."""
    import imexlb as im
    ran = 0
    for k, c, chunks, cfg, st, kw in _cases(dim):
        o = _oracle(dim, c, kw, st)
        init = (o.f.copy(), o.fb.copy(), o.p.copy(), o.u.copy())
        o.close()
        for prec in (im.FP16, im.FP32) + ((im.FIX64,) if c["rho0"] == 1.0 else ()):
            a = _run(cfg, st, im.FILL_FUSED, chunks, c["interv"], init, precision=prec)
            if a is None:
                break
            b = _run(cfg, st, im.FILL_KERNEL, chunks, c["interv"], init, precision=prec)
            what = "case %d %s precision %d" % (k, c, prec)
            assert_same(a[1], b[1], "Monitor, " + what)
            for name, x, y in zip(("f", "fb", "p", "u"), a[2], b[2]):
                assert_same(x, y, name + ", " + what)
            ran += 1
    assert ran >= N_CASES // 2
