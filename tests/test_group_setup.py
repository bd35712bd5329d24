"""Host setup of a multi-rank run (imexlb.GroupSetup: SetCartesian /
SetLocalLength boxes, each rank's geometry lists, PassInt across ranks, each
rank's obstacle scan and InitUP) against the oracle's rank group."""
import numpy as np
import pytest

CASES = [(2, 64, 32, 0, 2), (2, 64, 32, 0, 4), (2, 96, 40, 0, 3), (3, 24, 12, 12, 2), (3, 32, 16, 16, 4)]


def _both(case):
    import imexlb as im
    from oracle import orc
    dim, nx, ny, nz, P = case
    L = 0.125 if dim == 2 else 0.25
    cfg = im.make_config(dim, nx, ny, nz, charlength=L, xpos=0.25, re=20.0, ome=1.8)
    gs = im.GroupSetup(cfg, P, seed=500, allow_geom_error=True)
    og = orc.OracleGroup(orc.make_input(dim, nx, ny, nz, charlength=L, xpos=0.25, re=20.0, ome=1.8),
                         P, allow_geom_error=True)
    og.init_up(np.stack([rs.r_vec for rs in gs.ranks]))
    return im, gs, og


@pytest.mark.parametrize("case", CASES)
def test_group_setup_matches_oracle_ranks(built, case):
    im, gs, og = _both(case)
    dim = case[0]
    assert gs.np == og.np
    for r, (rs, o) in enumerate(zip(gs.ranks, og.ranks)):
        assert tuple(rs.cfg.local_length[:dim]) == o.local_length
        assert tuple(rs.cfg.local_start[:dim]) == o.start
        assert np.array_equal(rs.geo, o.geo)
        ol = o.lists
        for name in ("fluid_id", "bl", "br", "bu", "bd", "b_user"):
            assert np.array_equal(getattr(rs, name), ol[name]), (r, name)
        assert np.array_equal(rs.p, o.p) and np.array_equal(rs.u, o.u)


def test_decompose_agrees_with_oracle(built):
    import imexlb as im
    from oracle import orc
    for dim, gl in ((2, (65, 33)), (2, (1025, 513)), (3, (33, 17, 17)), (3, (257, 129, 129))):
        for P in (1, 2, 3, 4, 6, 8, 12, 16):
            assert im.decompose(dim, gl, P) == orc.decompose(dim, gl, P), (dim, gl, P)
