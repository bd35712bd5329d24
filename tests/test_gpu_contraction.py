"""GPU: the drop-in against a reference build that contracts a*b+c.

The oracle, and the bitwise FP64 kernel that is IEEE-equal to it, round
every operation once: the reference compiled without contraction. gfortran
and nvfortran contract a*b+c into fused multiply-adds by default on aarch64,
the Grace host of a GB300, and a reference built that way rounds
differently. The oracle's own source built with -ffp-contract=fast
(oracle/build.py, LIB_FMA) stands for that build. The test runs the D3Q27
sphere at 128x64x64 (the benchmark's flow, Re 100) for 1000 iterations with a
Monitor on every one in both oracle builds and on the GPU, and asserts that
the bitwise drop-in stays within the 1e-12 relative accuracy bar of the
contracting build: u (max-norm), the drag force and every Monitor value, and
p within 1e-14 of rho0/3 (p is the small deviation of the pressure from
rho0/3). On aarch64 it also asserts that the contracted build does round
differently; on a host whose baseline has no fused multiply-add the two
builds are the same.
"""
import os
import platform

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ITERS = 1000


def _rel_maxnorm(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def test_drop_in_within_the_bar_of_a_contracting_reference_build(built):
    import bench
    import imexlb as im
    from oracle import orc
    w = dict(bench.WORKLOADS["sphere_d3q27_128x64x64"])
    dim = w.pop("dim")
    nx, ny, nz = w.pop("nx"), w.pop("ny"), w.pop("nz")
    cfg = im.make_config(dim, nx, ny, nz, **w)
    st = im.Setup(cfg, seed=12345)
    inp = orc.make_input(dim, nx, ny, nz, charlength=w["charlength"], xpos=w["xpos"], re=w["re"],
                         ome=w["ome"], dt=w["dt"], rho0=w["rho0"])
    cores = os.cpu_count() or 1
    plain = orc.Oracle(inp, nthreads=cores)
    fused = orc.Oracle(inp, nthreads=cores, contract=True)
    try:
        for o in (plain, fused):
            o.init_up(st.r_vec)
            o.init_pdf()
        init = (plain.f.copy(), plain.fb.copy(), plain.p.copy(), plain.u.copy())
        log_p = plain.run(0, ITERS, 1)
        log_f = fused.run(0, ITERS, 1)
        F_f, _ = fused.forces()
        with im.Solver(cfg) as s:
            s.set_geometry(st)
            s.upload(*init)
            log_g = s.step(0, ITERS, 1)
            F_g, _ = s.observe()
            _, _, p, u = s.download(f=False, fb=False)
        # the bitwise kernel is the plain build, bit for bit
        assert np.array_equal(log_g.view(np.uint64), log_p.view(np.uint64))
        if platform.machine() == "aarch64":
            assert not np.array_equal(log_f.view(np.uint64), log_p.view(np.uint64)), \
                "the contracted build should round differently"
        ids = plain.lists["fluid_id"]
        err_u = _rel_maxnorm(u.reshape(-1, dim)[ids], fused.u.reshape(-1, dim)[ids])
        err_p = float(np.max(np.abs(p[ids] - fused.p[ids]))) / (w["rho0"] / 3.0)
        err_cd = abs(F_g[0] - F_f[0]) / abs(F_f[0])
        err_mon = float(np.max(np.abs(log_g - log_f) / log_f))
        print("GPU drop-in vs the contracting build after %d iterations (%s): u %.2e, p %.2e of "
              "rho0/3, drag %.2e, Monitor %.2e"
              % (ITERS, platform.machine(), err_u, err_p, err_cd, err_mon))
        assert err_u < 1e-12 and err_cd < 1e-12 and err_mon < 1e-12
        assert err_p < 1e-14
    finally:
        plain.close()
        fused.close()
