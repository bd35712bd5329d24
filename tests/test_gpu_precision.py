"""GPU: reduced-precision storage (FP32 / BF16 / FP16 populations, FP32
arithmetic), the fast FP64 option (minimal operation count with fused
multiply-adds) and the fixed-point kind (Q3.60 integers, integer arithmetic)
against the FP64 oracle.

These kinds are not bit-compatible with the reference; the checks are the
error budgets below after 300 iterations of a small cylinder / sphere flow:
relative L2 error of the velocity field over fluid nodes, relative error of
the obstacle force (drag), and the drift of the fluid mass sum relative to
the FP64 run's own mass scale.
"""
import numpy as np
import pytest

from parity_util import make_case

pytestmark = pytest.mark.gpu

# precision -> (max rel L2(u), max rel drag error)
BUDGET = {
    "fp64fast": (1e-12, 1e-11),
    "fix64": (1e-12, 1e-11),
    "fp32": (1e-5, 1e-5),
    "fp16": (5e-3, 1e-2),
    "bf16": (5e-2, 1e-1),
}


def _run(im, cfg, st, o, precision, steps):
    with im.Solver(cfg, precision=precision) as s:
        s.set_geometry(st)
        s.upload(o.f, o.fb, o.p, o.u)
        mon = s.step(0, steps, 50)
        F, m = s.observe()
        f, fb, p, u = s.download()
    return mon, F, m, u


@pytest.mark.parametrize("name", ["2d_64x32", "3d_32x16x16"])
@pytest.mark.parametrize("prec", sorted(BUDGET))
def test_reduced_precision_error_budget(built, name, prec):
    import imexlb as im
    steps = 300
    code = {"fp64fast": im.FP64_FAST, "fix64": im.FIX64, "fp32": im.FP32, "fp16": im.FP16,
            "bf16": im.BF16}[prec]
    cfg, st, o = make_case(name)
    mon, F, m, u = _run(im, cfg, st, o, code, steps)
    mon_ref = o.run(0, steps, 50)
    F_ref, _ = o.forces()
    m_ref = o.mass()
    ids = o.lists["fluid_id"]
    dim = cfg.dim
    uref = o.u.reshape(-1, dim)[ids]
    ug = u.reshape(-1, dim)[ids]
    l2 = np.linalg.norm(ug - uref) / np.linalg.norm(uref)
    drag = abs(F[0] - F_ref[0]) / abs(F_ref[0])
    mass_scale = np.abs(o.f.reshape(-1, o.s.nq)[ids]).sum()
    print("%s %s: rel L2(u) %.3e, rel drag err %.3e, mass diff/scale %.3e, Umax rel %.3e"
          % (name, prec, l2, drag, abs(m - m_ref) / mass_scale,
             np.max(np.abs(mon - mon_ref) / mon_ref)))
    tol_u, tol_f = BUDGET[prec]
    assert np.all(np.isfinite(u[ids * dim]))
    assert l2 < tol_u
    assert drag < tol_f
    assert np.allclose(mon, mon_ref, rtol=max(tol_u * 10, 1e-12), atol=0.0)


@pytest.mark.parametrize("prec", ["fp32", "fp16", "bf16", "fix64"])
def test_upload_download_roundtrip_rounds_once(built, prec):
    """A state uploaded into narrow storage and downloaded without stepping
    gives back f, p, u exactly (kept in FP64) and fb rounded once (for the
    fixed-point kind: to the nearest multiple of 2^-60)."""
    import imexlb as im
    code = {"fp32": im.FP32, "fp16": im.FP16, "bf16": im.BF16, "fix64": im.FIX64}[prec]
    cfg, st, o = make_case("2d_48x20_rho" if prec != "fix64" else "2d_64x32")
    rng = np.random.default_rng(0)
    fb0 = rng.uniform(-0.05, 0.05, o.fb.size)
    with im.Solver(cfg, precision=code) as s:
        s.set_geometry(st)
        s.upload(o.f, fb0, o.p, o.u)
        f, fb, p, u = s.download()
    assert np.array_equal(f, o.f) and np.array_equal(p, o.p) and np.array_equal(u, o.u)
    if prec == "fix64":
        # x -> the nearest multiple of 2^-60 (ties away from zero) -> the
        # nearest double (ties to even): both steps exact in numpy
        xi = fb0 * 2.0 ** 60
        a = np.abs(xi)
        v = np.where(a == np.floor(a), a, np.floor(a + 0.5)).astype(np.int64)
        want = np.sign(xi) * v.astype(np.float64) * 2.0 ** -60
        assert np.array_equal(fb, want)
        assert np.all(np.abs(fb - fb0) <= 2.0 ** -61 + 2.0 ** -53 * np.abs(fb0))
        return
    rel = {"fp32": 2.0 ** -24, "fp16": 2.0 ** -11, "bf16": 2.0 ** -8}[prec]
    assert np.all(np.abs(fb - fb0) <= rel * np.abs(fb0) + 1e-7)
