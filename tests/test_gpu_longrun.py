"""GPU: long runs against the oracle.

1. The FP64 drop-in on the D3Q27 sphere at the drop-in size (256x128x128,
   sphere diameter 24, Re 100: the input.in values bench.py uses for this
   lattice) for 1000 iterations (IMEXLB_LONGRUN_ITERS for another count) of
   the reference's loop (main.f90:48-63) with
   a Monitor on every one. The reference-rounding kernel must stay IEEE-equal
   to the oracle in every Monitor value and every element of f, fb, p and u;
   the fast FP64 kind (minimal operation count with fused multiply-adds) and
   the fixed-point kind (Q3.60 integers) must stay within 1e-12 relative in
   u (max-norm), the drag force and every Monitor value, the bar the drop-in's
   accuracy is stated at, and within 1e-14 of the pressure rho0/3 in p (the
   reference's p is the small deviation of the pressure from rho0/3; FP64
   sums of the 27 populations in another order already differ from the
   reference's by ~1e-12 of max|p| after 1000 iterations).
2. A batch of D2Q9 cylinder cases of different sizes and iteration budgets
   (FP32 storage, lockstep stepping) compared case by case with the FP64
   oracle, within an FP32 error budget.

The oracle runs threaded over the host cores (its node loops are
independent, so the thread count does not change its bits): about 85 s for
the 1000 sphere iterations on 16 cores.
"""
import os

import numpy as np
import pytest

from parity_util import same

pytestmark = pytest.mark.gpu

CHUNK = 1 << 24
# IMEXLB_LONGRUN_ITERS sets a longer run for the record (the oracle takes
# ~85 s per 1000 iterations on 16 cores)
ITERS = int(os.environ.get("IMEXLB_LONGRUN_ITERS", "1000"))


def _assert_same_chunked(a, b, what):
    assert a.shape == b.shape, what
    for lo in range(0, a.size, CHUNK):
        x, y = a[lo:lo + CHUNK], b[lo:lo + CHUNK]
        if np.array_equal(x.view(np.uint64), y.view(np.uint64)):
            continue
        ok = same(x, y)
        if not ok.all():
            bad = np.flatnonzero(~ok)
            raise AssertionError("%s differs at %d slots of chunk %d; first at %d: %r vs %r"
                                 % (what, bad.size, lo // CHUNK, lo + bad[0], x[bad[0]], y[bad[0]]))


def _rel_maxnorm(a, b):
    fin = np.isfinite(b)
    assert np.array_equal(np.isfinite(a), fin)
    return float(np.max(np.abs(a[fin] - b[fin])) / np.max(np.abs(b[fin])))


def test_sphere_1000_iterations_against_oracle(built):
    import bench
    import imexlb as im
    from oracle import orc
    w = dict(bench.WORKLOADS["sphere_d3q27_256x128x128"])
    dim = w.pop("dim")
    nx, ny, nz = w.pop("nx"), w.pop("ny"), w.pop("nz")
    cfg = im.make_config(dim, nx, ny, nz, **w)
    st = im.Setup(cfg, seed=12345)
    o = orc.Oracle(orc.make_input(dim, nx, ny, nz, charlength=w["charlength"], xpos=w["xpos"],
                                  re=w["re"], ome=w["ome"], dt=w["dt"], rho0=w["rho0"]),
                   nthreads=os.cpu_count() or 1)
    try:
        o.init_up(st.r_vec)
        o.init_pdf()
        f0, fb0, p0, u0 = o.f.copy(), o.fb.copy(), o.p.copy(), o.u.copy()
        log_o = o.run(0, ITERS, 1)
        F_o, _ = o.forces()
        ids = o.lists["fluid_id"]

        with im.Solver(cfg) as s:
            s.set_geometry(st)
            s.upload(f0, fb0, p0, u0)
            log_g = s.step(0, ITERS, 1)
            assert log_g.size == ITERS
            _assert_same_chunked(log_g, log_o, "Monitor")
            F_g, _ = s.observe()
            for name, flags, ref in (("p", dict(f=False, fb=False, u=False), o.p),
                                     ("u", dict(f=False, fb=False, p=False), o.u),
                                     ("f", dict(fb=False, p=False, u=False), o.f),
                                     ("fb", dict(f=False, p=False, u=False), o.fb)):
                got = [a for a in s.download(**flags) if a is not None][0]
                _assert_same_chunked(got, ref, name)
                del got
        # the force sums of the two sides agree to double-double rounding
        fbv = o.fb.reshape(-1, o.s.nq)
        assert np.all(np.abs(F_g - F_o) <= 4.5e-16 * 2 * np.abs(fbv[ids]).sum())

        for kind, name in ((im.FP64_FAST, "FP64 fast"), (im.FIX64, "fixed point")):
            with im.Solver(cfg, precision=kind) as s:
                s.set_geometry(st)
                s.upload(f0, fb0, p0, u0)
                log_k = s.step(0, ITERS, 1)
                F_k, _ = s.observe()
                _, _, p, u = s.download(f=False, fb=False)
            err_p = _rel_maxnorm(p[ids], o.p[ids])
            # p is the deviation of the pressure from rho0/3 (sum f / 3 of the
            # deviations f): relative to the pressure itself
            err_p_abs = float(np.max(np.abs(p[ids] - o.p[ids]))) / (w["rho0"] / 3.0)
            err_u = _rel_maxnorm(u.reshape(-1, dim)[ids], o.u.reshape(-1, dim)[ids])
            err_cd = abs(F_k[0] - F_o[0]) / abs(F_o[0])
            err_mon = float(np.max(np.abs(log_k - log_o) / log_o))
            print("%s after %d iterations: p %.2e of max|p| (%.2e of rho0/3), u %.2e, Cd %.2e, "
                  "Monitor %.2e" % (name, ITERS, err_p, err_p_abs, err_u, err_cd, err_mon))
            assert err_u < 1e-12 and err_cd < 1e-12 and err_mon < 1e-12, name
            # the pressure deviation is ~1e-3 of rho0/3: summed in another
            # order, FP64 itself differs from the reference by ~1e-12 of it
            assert err_p_abs < 1e-14 and err_p < 5e-12, name
    finally:
        o.close()


# nx, ny, charlength (fraction of nx), Re, iteration budget after the first
BATCH = [(64, 32, 0.25, 40.0, 300), (48, 24, 0.3, 60.0, 170), (80, 40, 0.2, 100.0, 230)]
# FP32 budget (rel. L2 of u over fluid nodes, rel. drag error): the drag
# bound is looser (the momentum-exchange sum cancels: FP32 storage measures
# 1.9e-5 on the Re 40 case, 6.5e-5 on a Re 150 case)
FP32_BUDGET = (1e-5, 2e-4)


def test_batch_cases_against_oracle(built):
    import imexlb as im
    from oracle import orc
    solvers, oracles = [], []
    try:
        for nx, ny, L, re, _ in BATCH:
            nu = 0.05 * L * nx / re
            ome = 1.0 / (3.0 * nu + 0.5)
            args = dict(charlength=L, xpos=0.25, re=re, ome=ome, dt=1.0, rho0=1.0)
            cfg = im.make_config(2, nx, ny, **args)
            st = im.Setup(cfg)
            o = orc.Oracle(orc.make_input(2, nx, ny, **args))
            o.init_up(st.r_vec)
            o.init_pdf()
            s = im.Solver(cfg, precision=im.FP32)
            s.set_geometry(st)
            s.upload(o.f, o.fb, o.p, o.u)
            s.step(0, 1)  # a batch member has taken one iteration on its own
            solvers.append(s)
            oracles.append(o)
        budgets = [b[-1] for b in BATCH]
        with im.Batch(solvers) as b:
            b.step(steps=budgets)
        for (nx, ny, L, re, n), s, o in zip(BATCH, solvers, oracles):
            o.run(0, 1 + n, 0)
            F, _ = s.observe()
            _, _, _, u = s.download(f=False, fb=False, p=False)
            F_o, _ = o.forces()
            ids = o.lists["fluid_id"]
            ug, uo = u.reshape(-1, 2)[ids], o.u.reshape(-1, 2)[ids]
            l2 = np.linalg.norm(ug - uo) / np.linalg.norm(uo)
            drag = abs(F[0] - F_o[0]) / abs(F_o[0])
            print("batch case %dx%d Re %g after %d: rel L2(u) %.2e, drag %.2e"
                  % (nx, ny, re, 1 + n, l2, drag))
            assert l2 < FP32_BUDGET[0] and drag < FP32_BUDGET[1]
    finally:
        for s in solvers:
            s.close()
        for o in oracles:
            o.close()
