"""GPU parity at the benchmark's full lattice sizes.

The small parity cases pin the arithmetic; these run the same comparison on
the workloads bench.py times (D2Q9 1024x512, D3Q27 256x128x128 and
512x256x256, FP64 with the reference's rounding): a few iterations with a
Monitor on every one, then f, fb, p and u compared with the oracle element by
element (IEEE equality, NaN matching NaN). The oracle runs threaded over the
host cores (its node loops are independent, so the thread count does not
change its bits), which keeps the largest case to seconds per iteration.
Arrays are compared in chunks to bound the host memory beside the two copies
of the state.
"""
import os

import numpy as np
import pytest

from parity_util import same

pytestmark = pytest.mark.gpu

CHUNK = 1 << 24


def _assert_same_chunked(a, b, what):
    assert a.shape == b.shape, what
    for lo in range(0, a.size, CHUNK):
        x, y = a[lo:lo + CHUNK], b[lo:lo + CHUNK]
        if np.array_equal(x.view(np.uint64), y.view(np.uint64)):
            continue
        ok = same(x, y)
        if not ok.all():
            bad = np.flatnonzero(~ok)
            i = bad[0]
            raise AssertionError("%s differs at %d slots of chunk %d; first at %d: %r vs %r"
                                 % (what, bad.size, lo // CHUNK, lo + i, x[i], y[i]))


def _case(workload):
    import bench
    import imexlb as im
    from oracle import orc
    w = dict(bench.WORKLOADS[workload])
    dim = w.pop("dim")
    nx, ny, nz = w.pop("nx"), w.pop("ny"), w.pop("nz")
    cfg = im.make_config(dim, nx, ny, nz, **w)
    st = im.Setup(cfg, seed=12345)
    o = orc.Oracle(orc.make_input(dim, nx, ny, nz, charlength=w["charlength"], xpos=w["xpos"],
                                  re=w["re"], ome=w["ome"], dt=w["dt"], rho0=w["rho0"]),
                   nthreads=os.cpu_count() or 1)
    o.init_up(st.r_vec)
    o.init_pdf()
    return cfg, st, o


def _run_and_compare(cfg, st, o, steps, fill):
    import imexlb as im
    with im.Solver(cfg) as s:
        s.set_geometry(st)
        s.set_fill_mode(fill)
        s.upload(o.f, o.fb, o.p, o.u)
        log_g = s.step(0, steps, 1)
        log_o = o.run(0, steps, 1)
        assert log_g.size == steps
        _assert_same_chunked(log_g, log_o, "Monitor")
        # one array at a time: the largest case holds 7.75 GB per array
        for name, flags, ref in (("p", dict(f=False, fb=False, u=False), o.p),
                                 ("u", dict(f=False, fb=False, p=False), o.u),
                                 ("f", dict(fb=False, p=False, u=False), o.f),
                                 ("fb", dict(f=False, p=False, u=False), o.fb)):
            got = [a for a in s.download(**flags) if a is not None][0]
            _assert_same_chunked(got, ref, name)
            del got


@pytest.mark.parametrize("workload,steps", [("cylinder_d2q9_1024x512", 6),
                                            ("sphere_d3q27_256x128x128", 3)])
def test_benchmark_sizes_match_oracle(built, workload, steps):
    import imexlb as im
    cfg, st, o = _case(workload)
    try:
        _run_and_compare(cfg, st, o, steps, im.FILL_FUSED)
    finally:
        o.close()


def test_benchmark_size_separate_fill_matches_oracle(built):
    import imexlb as im
    cfg, st, o = _case("sphere_d3q27_256x128x128")
    try:
        _run_and_compare(cfg, st, o, 2, im.FILL_KERNEL)
    finally:
        o.close()


def test_largest_sphere_matches_oracle(built):
    """D3Q27 512x256x256 (33.9M nodes; the reduced-precision study's FP64 run)."""
    import imexlb as im
    cfg, st, o = _case("sphere_d3q27_512x256x256")
    try:
        _run_and_compare(cfg, st, o, 2, im.FILL_FUSED)
    finally:
        o.close()
