"""GPU: the persistent ensemble kernel (IMEXLB_BATCH_PERSISTENT).

One cooperative launch per call runs every iteration of every case, each
case's iteration n waiting (with a bounded wait) for its own iteration n-1's
boundary copies. Checked against lockstep stepping of the same cases (same
FP32 formulas; the tolerance allows for different fused-multiply-add choices
of the two kernels), against the FP64 oracle case by case (an FP32 error
budget: rel. L2 of u 1e-5, drag 2e-4), and with a wait that is made to run out: the call
returns IMEXLB_ERR_TIMEOUT and the device stays usable. The stall is a count
nothing reaches, set on the host; no kernel faults.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = [  # nx, ny, L (fraction of nx), Re, y offset
    (64, 32, 0.25, 40.0, 0.0),
    (48, 24, 0.3, 60.0, 1.5),
    (80, 40, 0.2, 100.0, -2.0),
    (96, 48, 0.2, 150.0, 0.5),
]


def _solver(im, nx, ny, L, re, yoff, precision=None):
    nu = 0.05 * L * nx / re
    ome = 1.0 / (3.0 * nu + 0.5)
    cfg = im.make_config(2, nx, ny, charlength=L, xpos=0.25, re=re, ome=ome, yoff=yoff)
    st = im.Setup(cfg)
    s = im.Solver(cfg, precision=im.FP32 if precision is None else precision)
    s.set_geometry(st)
    s.upload(st.f, st.fb, st.p, st.u)
    s.init_pdf()
    s.step(0, 1)
    return s


def _close(a, b, rel=2e-6):
    fin = np.isfinite(b)
    assert np.array_equal(np.isfinite(a), fin)
    scale = np.abs(b[fin]).max()
    assert np.abs(a[fin] - b[fin]).max() <= rel * scale


@pytest.mark.parametrize("prec", ["fp32", "fp16"])
def test_persistent_matches_lockstep(built, prec):
    import imexlb as im
    code = {"fp32": im.FP32, "fp16": im.FP16}[prec]
    calls = [[40, 17, 0, 25], [3, 30, 22, 1], [0, 0, 9, 0]]
    results = []
    for mode in (im.BATCH_LOCKSTEP, im.BATCH_PERSISTENT):
        ss = [_solver(im, *c, precision=code) for c in CASES]
        with im.Batch(ss) as b:
            b.set_mode(mode)
            for steps in calls:
                b.step(steps=steps)
        results.append([s.download() for s in ss])
        for s in ss:
            s.close()
    rel = 2e-6 if prec == "fp32" else 2e-3
    for got, ref in zip(results[1], results[0]):
        for a, r in zip(got, ref):
            _close(a, r, rel)


def test_persistent_cases_against_oracle(built):
    import imexlb as im
    from oracle import orc
    budgets = [300, 170, 230, 120]
    solvers, oracles = [], []
    try:
        for (nx, ny, L, re, _), n in zip(CASES, budgets):
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
            s.step(0, 1)
            solvers.append(s)
            oracles.append(o)
        with im.Batch(solvers) as b:
            b.set_mode(im.BATCH_PERSISTENT)
            b.step(steps=budgets)
        for n, s, o in zip(budgets, solvers, oracles):
            o.run(0, 1 + n, 0)
            F, _ = s.observe()
            _, _, _, u = s.download(f=False, fb=False, p=False)
            F_o, _ = o.forces()
            ids = o.lists["fluid_id"]
            ug, uo = u.reshape(-1, 2)[ids], o.u.reshape(-1, 2)[ids]
            l2 = np.linalg.norm(ug - uo) / np.linalg.norm(uo)
            drag = abs(F[0] - F_o[0]) / abs(F_o[0])
            assert l2 < 1e-5 and drag < 2e-4, (l2, drag)
    finally:
        for s in solvers:
            s.close()
        for o in oracles:
            o.close()


def test_persistent_wait_runs_out(built):
    """A case whose step tiles wait for a count nothing reaches: the wait
    gives up after its budget, every block returns, the call reports
    IMEXLB_ERR_TIMEOUT naming the case, and the device keeps working."""
    import time
    import imexlb as im
    L = im.lib()
    ss = [_solver(im, *c) for c in CASES]
    with im.Batch(ss) as b:
        b.set_mode(im.BATCH_PERSISTENT)
        assert L.imexlb_testing_batch_stall(b.b, 2, 0.05) == im.IMEXLB_OK
        t0 = time.perf_counter()
        with pytest.raises(im.ImexlbError) as ei:
            b.step(nsteps=20)
        elapsed = time.perf_counter() - t0
        assert ei.value.code == im.ERR_TIMEOUT
        assert "case 2" in str(ei.value)
        assert elapsed < 5.0
    for s in ss:
        s.close()
    # the context is intact: a fresh batch and a single handle step normally
    ss = [_solver(im, *c) for c in CASES]
    with im.Batch(ss) as b:
        b.set_mode(im.BATCH_PERSISTENT)
        b.step(nsteps=10)
    for s in ss:
        _, _, _, u = s.download()
        assert np.all(np.isfinite(u))
        s.close()
