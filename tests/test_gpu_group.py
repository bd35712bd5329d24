"""GPU: a multi-rank run (imexlb_group_*) against the oracle's rank group,
bit for bit: Monitor (maximum over ranks), and every rank's f, fb, p, u."""
import numpy as np
import pytest

from parity_util import assert_same

pytestmark = pytest.mark.gpu

CASES = [(2, 64, 32, 0, 2), (2, 64, 32, 0, 4), (2, 96, 40, 0, 3), (3, 24, 12, 12, 2),
         (3, 32, 16, 16, 4)]


def _setup(case):
    import imexlb as im
    from oracle import orc
    dim, nx, ny, nz, P = case
    L = 0.125 if dim == 2 else 0.25
    cfg = im.make_config(dim, nx, ny, nz, charlength=L, xpos=0.25, re=20.0, ome=1.8)
    gs = im.GroupSetup(cfg, P, seed=900, allow_geom_error=True)
    og = orc.OracleGroup(orc.make_input(dim, nx, ny, nz, charlength=L, xpos=0.25, re=20.0, ome=1.8),
                         P, allow_geom_error=True)
    og.init_up(np.stack([rs.r_vec for rs in gs.ranks]))
    og.init_pdf()
    return im, gs, og


@pytest.mark.parametrize("case", CASES)
def test_group_matches_oracle_group(built, case):
    im, gs, og = _setup(case)
    solvers = []
    try:
        for rs, o in zip(gs.ranks, og.ranks):
            s = im.Solver(rs.cfg)
            s.set_geometry(rs)
            s.upload(o.f, o.fb, o.p, o.u)
            solvers.append(s)
        with im.Group(solvers) as g:
            logs = [g.step(0, 9, 4), g.step(9, 21, 4)]
            log_o = og.run(0, 30, 4)
            assert_same(np.concatenate(logs), log_o, "Monitor")
            for r, (s, o) in enumerate(zip(solvers, og.ranks)):
                f, fb, p, u = s.download()
                assert_same(f, o.f, "rank %d f" % r)
                assert_same(fb, o.fb, "rank %d fb" % r)
                assert_same(p, o.p, "rank %d p" % r)
                assert_same(u, o.u, "rank %d u" % r)
    finally:
        for s in solvers:
            s.close()


def test_group_init_pdf_on_device_and_rank_rules(built):
    case = (2, 64, 32, 0, 2)
    im, gs, og = _setup(case)
    solvers = []
    try:
        for rs in gs.ranks:
            s = im.Solver(rs.cfg)
            s.set_geometry(rs)
            s.upload(rs.f, rs.fb, rs.p, rs.u)
            s.init_pdf()
            solvers.append(s)
        with pytest.raises(im.ImexlbError):  # a rank is stepped by its group
            solvers[0].step(0, 1)
        with pytest.raises(im.ImexlbError):  # ranks out of MPI order
            im.Group(solvers[::-1])
        with im.Group(solvers) as g:
            log = g.step(0, 12, 5)
            assert_same(log, og.run(0, 12, 5), "Monitor")
            for s, o in zip(solvers, og.ranks):
                f, fb, p, u = s.download()
                assert_same(f, o.f, "f")
                assert_same(u, o.u, "u")
    finally:
        for s in solvers:
            s.close()


def test_group_ranks_keep_the_separate_fill(built):
    """The ranks of a group run the group's copy program (PassF across
    ranks): no fused boundary plan, and asking for one is refused."""
    im, gs, og = _setup((2, 64, 32, 0, 2))
    solvers = []
    try:
        for rs in gs.ranks:
            s = im.Solver(rs.cfg)
            s.set_geometry(rs)
            solvers.append(s)
            assert s.fill_mode() == im.FILL_KERNEL
            with pytest.raises(im.ImexlbError) as e:
                s.set_fill_mode(im.FILL_FUSED)
            assert e.value.code == im.ERR_UNSUPPORTED
    finally:
        for s in solvers:
            s.close()
