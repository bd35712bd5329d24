"""The corrected-physics obstacle rule (imexlb_host_obstacle_cells), a mode
apart from the reference: every interior solid cell with a fluid neighbour
(proper e_x + dy*e_y + dz*e_z offsets) is an obstacle cell, instead of the
reference's first cell per x-row found by the odd probe
geo(id + e_x + dy*(iq*dim+1)) (initialization.f90:232-253).

The library's rule is checked against the oracle's own restatement, against
its definition, and by its purpose: every solid slot a fluid node pulls is
written by the boundary program (in the reference rule most are not, and
those nodes pull the never-written zero of a solid cell)."""
import numpy as np
import pytest

CASES = [(2, 64, 32, 0, 0.25, 0.3), (2, 96, 40, 0, 0.2, 0.25), (3, 32, 16, 16, 0.25, 0.3)]


def _cfg(im, dim, nx, ny, nz, L, xp):
    return im.make_config(dim, nx, ny, nz, charlength=L, xpos=xp, re=20.0, ome=1.8)


def _interior_ids(cfg):
    G = 3
    dim = cfg.dim
    xs = np.arange(cfg.nx + 1) + G
    ys = np.arange(cfg.ny + 1) + G
    if dim == 2:
        return (xs[None, :] + cfg.dy * ys[:, None]).ravel()
    zs = np.arange(cfg.nz + 1) + G
    return (xs[None, None, :] + cfg.dy * ys[None, :, None] + cfg.dz * zs[:, None, None]).ravel()


def _offsets(im, dim):
    t, e = im.lattice(dim)
    return e.reshape(-1, dim)


@pytest.mark.parametrize("case", CASES)
def test_library_and_oracle_lists_agree(built, case):
    import imexlb as im
    from oracle import orc
    dim, nx, ny, nz, L, xp = case
    st = im.Setup(_cfg(im, *case), physics="corrected")
    o = orc.Oracle(orc.make_input(dim, nx, ny, nz, charlength=L, xpos=xp, re=20.0, ome=1.8),
                   allow_geom_error=True)
    o.use_corrected_obstacles()
    assert np.array_equal(st.b_user, o.lists["b_user"])
    assert len(st.b_user) > 0


@pytest.mark.parametrize("case", CASES)
def test_list_is_every_wetted_solid_cell_in_scan_order(built, case):
    import imexlb as im
    cfg = _cfg(im, *case)
    st = im.Setup(cfg, physics="corrected")
    dim = cfg.dim
    e = _offsets(im, dim)
    off = e[:, 0] + cfg.dy * e[:, 1] + (cfg.dz * e[:, 2] if dim == 3 else 0)
    ids = _interior_ids(cfg)
    solid = ids[st.geo[ids] == 0]
    wet = np.array([np.any(st.geo[s + off] == 1) for s in solid], dtype=bool)
    assert np.array_equal(st.b_user, solid[wet])  # x fastest, like the scan


@pytest.mark.parametrize("physics,case", [("reference", CASES[0]), ("corrected", CASES[0]),
                                          ("reference", CASES[1]), ("corrected", CASES[1])])
def test_every_pulled_solid_slot_is_written(built, physics, case):
    import imexlb as im
    cfg = _cfg(im, *case)
    st = im.Setup(cfg, physics=physics)
    d = im.make_desc(cfg)
    nq, dim = cfg.nq, cfg.dim
    lists = {k: getattr(st, k) for k in ("fluid_id", "bl", "br", "bu", "bd", "b_user")}
    slots = np.arange(cfg.array_size * nq, dtype=np.float64)
    src, _ = im.resolve_bc(d, lists, slots)
    e = _offsets(im, dim)
    off = e[:, 0] + cfg.dy * e[:, 1] + (cfg.dz * e[:, 2] if dim == 3 else 0)
    interior = np.zeros(cfg.array_size, dtype=bool)
    interior[_interior_ids(cfg)] = True
    stale = 0
    pulled = 0
    for x in st.fluid_id:
        for q in range(nq):
            s = x - off[q]  # the cell fluid node x pulls direction q from
            if interior[s] and st.geo[s] == 0:
                pulled += 1
                slot = s * nq + q
                stale += int(src[slot] == slot)  # never written by the copies
    assert pulled > 0
    if physics == "corrected":
        assert stale == 0
    else:
        assert stale > 0  # the reference leaves most solid links unbounced
