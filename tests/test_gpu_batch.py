"""GPU: ensembles stepped in lockstep (imexlb_batch_*) and field sampling.

A batch of cases of different sizes and iteration budgets must give, case by
case, the same state as stepping each handle on its own (same FP32 formulas;
the tolerance allows for different fused-multiply-add choices in the two
kernels). The sampler must equal a bilinear sample of the downloaded p, u.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = [  # nx, ny, L (fraction of nx), Re, y offset
    (64, 32, 0.25, 40.0, 0.0),
    (48, 24, 0.3, 60.0, 1.5),
    (80, 40, 0.2, 100.0, -2.0),
]


def _solver(im, nx, ny, L, re, yoff):
    nu = 0.05 * L * nx / re
    ome = 1.0 / (3.0 * nu + 0.5)
    cfg = im.make_config(2, nx, ny, charlength=L, xpos=0.25, re=re, ome=ome, yoff=yoff)
    st = im.Setup(cfg)
    s = im.Solver(cfg, precision=im.FP32)
    s.set_geometry(st)
    s.upload(st.f, st.fb, st.p, st.u)
    s.init_pdf()
    s.step(0, 1)
    return s


def test_batch_matches_individual_stepping(built):
    import imexlb as im
    budgets = [40, 17, 33]
    alone = [_solver(im, *c) for c in CASES]
    for s, n in zip(alone, budgets):
        s.step(1, n)
    ref = [s.download() for s in alone]
    grouped = [_solver(im, *c) for c in CASES]
    with im.Batch(grouped) as b:
        b.step(steps=budgets[:1] + [9, 9])     # two calls, unequal budgets
        b.step(steps=[0, budgets[1] - 9, budgets[2] - 9])
    for s, r in zip(grouped, ref):
        got = s.download()
        for a, bb in zip(got, r):
            fin = np.isfinite(bb)
            assert np.array_equal(np.isfinite(a), fin)
            scale = np.abs(bb[fin]).max()
            assert np.abs(a[fin] - bb[fin]).max() <= 2e-6 * scale
    # stepping can continue on the handles after a batch call
    grouped[0].step(41, 3)


def test_batch_tune_picks_a_shape(built):
    import imexlb as im
    ss = [_solver(im, *c) for c in CASES]
    with im.Batch(ss) as b:
        shape = b.tune(trial=3)
        assert 0 <= shape < 6
        b.step(nsteps=12)
    for s in ss:
        f, fb, p, u = s.download()
        assert np.all(np.isfinite(u))


def test_sample_is_bilinear_of_the_state(built):
    import imexlb as im
    s = _solver(im, 64, 32, 0.25, 40.0, 0.0)
    s.step(1, 10)
    W, H = 20, 9
    smp = s.sample(W, H)
    _, _, p, u = s.download()
    cfg_dy = 64 + 1 + 6
    L0, L1 = 65, 33
    node = lambda x, y: (x + 3) + cfg_dy * (y + 3)
    fluid = np.zeros((L1, L0))
    P = np.zeros((L1, L0))
    UX = np.zeros((L1, L0))
    UY = np.zeros((L1, L0))
    fid = set(s._keep[1]["fluid_id"].tolist())
    for y in range(L1):
        for x in range(L0):
            i = node(x, y)
            if i in fid:
                fluid[y, x], P[y, x], UX[y, x], UY[y, x] = 1.0, p[i], u[2 * i], u[2 * i + 1]
    for j in range(H):
        for i in range(W):
            X = min(max((i + 0.5) * L0 / W - 0.5, 0), L0 - 1)
            Y = min(max((j + 0.5) * L1 / H - 0.5, 0), L1 - 1)
            x0, y0 = min(int(X), L0 - 2), min(int(Y), L1 - 2)
            fx, fy = X - x0, Y - y0
            for k, F in enumerate((fluid, P, UX, UY)):
                v = ((1 - fy) * ((1 - fx) * F[y0, x0] + fx * F[y0, x0 + 1]) +
                     fy * ((1 - fx) * F[y0 + 1, x0] + fx * F[y0 + 1, x0 + 1]))
                assert abs(smp[k, j, i] - v) <= 1e-5 * max(1.0, abs(v)), (k, i, j)
