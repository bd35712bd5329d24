"""The fused boundary plan (IMEXLB_FILL_FUSED), checked on the host.

imexlb_testing_fused_pull emulates one step's pulls two ways on arbitrary
slot values: with the resolved BoundaryCondition copies (lbm.f90:96-155,
lbm_3d.f90:96-157) written first and a plain pull, and with the plan the
fused step kernel follows (closed forms on the inlet, outlet, wall and
periodic faces; source rows elsewhere; obstacle copies by the node that
writes their source). Every fluid node must pull the same value in every
direction."""
import numpy as np
import pytest

CASES = [(2, 64, 32, 0, 0.125, 0.25), (2, 48, 20, 0, 0.2, 0.3), (2, 30, 31, 0, 0.3, 0.5),
         (3, 32, 16, 16, 0.25, 0.25), (3, 24, 12, 14, 0.3, 0.35), (3, 20, 9, 11, 0.4, 0.5)]


def _lists(st):
    return {k: getattr(st, k) for k in ("fluid_id", "bl", "br", "bu", "bd", "b_user")}


def _check(im, cfg, lists, seed=0, expect_fused=True):
    d = im.make_desc(cfg)
    rng = np.random.default_rng(seed)
    n = cfg.array_size * cfg.nq
    cur, prev = rng.standard_normal(n), rng.standard_normal(n)
    a, b, nrec = im.fused_pull(d, lists, cur, prev)
    if not expect_fused:
        assert b is None
        return nrec
    assert b is not None
    fl = np.asarray(lists["fluid_id"])
    sel = (np.arange(cfg.nq)[:, None] * cfg.array_size + fl[None, :]).ravel()
    assert np.count_nonzero(a[sel]) == sel.size  # every fluid pull was emulated
    assert np.array_equal(a, b)
    return nrec


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("physics", ["reference", "corrected"])
def test_fused_pulls_equal_the_copy_program(built, case, physics):
    import imexlb as im
    dim, nx, ny, nz, L, xp = case
    cfg = im.make_config(dim, nx, ny, nz, charlength=L, xpos=xp, re=20.0, ome=1.8)
    st = im.Setup(cfg, seed=2, physics=physics)
    nrec = _check(im, cfg, _lists(st))
    # records only on the box's edges and next to the obstacle, not on faces
    edges = 4 * ((nx + 1) + (ny + 1) + (nz + 1)) if dim == 3 else 4
    assert 0 < nrec <= edges + (125 if dim == 3 else 25) * len(st.b_user)


def test_records_stay_few_on_a_large_lattice(built):
    import imexlb as im
    cfg = im.make_config(3, 96, 48, 40, charlength=0.125, xpos=0.25, re=50.0, ome=1.8)
    st = im.Setup(cfg, seed=5)
    nrec = _check(im, cfg, _lists(st), seed=3)
    # 12 edges of the box plus the cells around the sphere
    assert nrec < 4 * (97 + 49 + 41) + 60 * len(st.b_user)


def test_obstacle_next_to_a_wall_keeps_the_separate_program(built):
    """A ghost slot that copies an obstacle slot before the obstacle copies
    rewrite it holds a value of the previous iteration: no plan."""
    import imexlb as im
    cfg = im.make_config(2, 64, 32, 0, charlength=0.125, xpos=0.25, re=20.0, ome=1.8)
    st = im.Setup(cfg, seed=1)
    lists = {k: v.copy() for k, v in _lists(st).items()}
    cell = (20 + 3) + cfg.dy * (1 + 3)  # x = 20, y = 1
    lists["fluid_id"] = lists["fluid_id"][lists["fluid_id"] != cell]
    lists["b_user"] = np.sort(np.append(lists["b_user"], cell))
    _check(im, cfg, lists, expect_fused=False)


def test_obstacle_touching_the_inlet_column(built):
    """Obstacle cells in the first interior column: the inlet copies read
    their slots after the obstacle copies wrote them."""
    import imexlb as im
    cfg = im.make_config(2, 40, 24, 0, charlength=0.125, xpos=0.25, re=20.0, ome=1.8)
    st = im.Setup(cfg, seed=1)
    lists = {k: v.copy() for k, v in _lists(st).items()}
    cells = [(0 + 3) + cfg.dy * (y + 3) for y in (10, 11, 12)] + [(1 + 3) + cfg.dy * (11 + 3)]
    for c in cells:
        lists["fluid_id"] = lists["fluid_id"][lists["fluid_id"] != c]
    lists["b_user"] = np.sort(np.concatenate([lists["b_user"], cells]))
    _check(im, cfg, lists, seed=4)


def _random_geometry(im, rng, dim, wall_margin=0):
    """A small lattice with a few random obstacle blobs anywhere in it (also
    against the walls, the inlet and the outlet), or at least `wall_margin`
    nodes from the walls (the wall axis: y in 2D, z in 3D)."""
    n = (int(rng.integers(12, 40)), int(rng.integers(8, 24)), 0) if dim == 2 else \
        (int(rng.integers(10, 20)), int(rng.integers(6, 12)), int(rng.integers(6, 12)))
    cfg = im.make_config(dim, *n, charlength=0.2, xpos=0.5, re=20.0, ome=1.8)
    st = im.Setup(cfg, seed=int(rng.integers(1 << 30)))
    geo = st.geo.copy()
    lists = {k: getattr(st, k).copy() for k in ("fluid_id", "bl", "br", "bu", "bd", "b_user")}
    L = [n[0] + 1, n[1] + 1, n[2] + 1]
    cells = set()
    w = dim - 1  # wall axis
    for _ in range(int(rng.integers(1, 4))):
        c = [int(rng.integers(0, L[k])) for k in range(dim)]
        r = [int(rng.integers(0, 3)) for _ in range(dim)]
        rng_k = [range(max(0, c[k] - r[k]), min(L[k], c[k] + r[k] + 1)) for k in range(dim)]
        rng_k[w] = range(max(rng_k[w].start, wall_margin), min(rng_k[w].stop, L[w] - wall_margin))
        for x in rng_k[0]:
            for y in rng_k[1]:
                for z in (rng_k[2] if dim == 3 else [0]):
                    cells.add((x + 3) + cfg.dy * (y + 3) + (cfg.dz * (z + 3) if dim == 3 else 0))
    cells = np.array(sorted(c for c in cells if geo[c] == 1), dtype=np.int64)
    keep = ~np.isin(lists["fluid_id"], cells)
    if keep.sum() < 8:
        return None
    geo[cells] = 0
    lists["fluid_id"] = lists["fluid_id"][keep]
    lists["b_user"] = np.unique(np.concatenate([lists["b_user"], cells])).astype(lists["b_user"].dtype)
    return cfg, lists


@pytest.mark.parametrize("dim", [2, 3])
def test_random_obstacles_plan_or_refuse(built, dim):
    """Random obstacle blobs: every plan the host accepts pulls exactly what
    the copy program gives (the host refuses a plan, and keeps the separate
    kernel, for geometries such as an obstacle right inside a wall)."""
    import imexlb as im
    rng = np.random.default_rng(1000 + dim)
    planned = refused = 0
    for trial in range(40 if dim == 2 else 24):
        g = _random_geometry(im, rng, dim, wall_margin=3 if trial % 2 else 0)
        if g is None:
            continue
        cfg, lists = g
        d = im.make_desc(cfg)
        n = cfg.array_size * cfg.nq
        cur, prev = rng.standard_normal(n), rng.standard_normal(n)
        try:
            a, b, nrec = im.fused_pull(d, lists, cur, prev)
        except im.ImexlbError:
            continue  # the geometry itself is rejected (a pulled slot read outside the arrays)
        if b is None:
            refused += 1
            continue
        planned += 1
        assert np.array_equal(a, b), "trial %d" % trial
    assert planned >= (10 if dim == 2 else 6)
