"""GPU: what the trained warm-start network gains over the method without it.

Reduced case of the learned warm start: the network (imexlb.neural, trained
with the library's tcgen05 kernels) learns from an ensemble of 64 cylinder
flows on a 256 x 128 lattice (FP32 storage, lockstep batch, time means of
the last third of 60 nx iterations), then predicts (p, u) for 8 held-out
seeds. Each held-out case runs twice in FP64 from the same code path: from
rest, as the plain uniform-initialised LBM, and from the prediction (f = feq
of the predicted p, u). The plain run is the arbiter: the mean drag of its last
quarter is the converged Cd, and a run has converged at the first
checkpoint after which its trailing mean Cd (1000 iterations) stays within
1 % of that value to the end. Steady wakes (Re 20-45) isolate the transient
the prediction removes; vortex shedding (Re > ~47) has to grow from the
perturbation either way.

The reference's own initial state is InitUP (initialization.f90:259-282),
the plain LBM's transient starts from it; the prediction replaces it.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_trained_network_shortens_the_transient(built):
    from imexlb import warmstart as ws
    net, info = ws.train_network(ncases=64, nx_range=(256, 256), nx_iters=60, train_steps=1500,
                                 d_range=(16.0, 32.0), re_range=(20.0, 200.0))
    assert info["loss_last"] < 0.25 * info["loss_first"]
    rows = ws.evaluate(net, range(1000, 1008), steps=40000, every=10, nx=256, log=lambda r: None,
                       d_range=(16.0, 32.0), re_range=(20.0, 45.0), warm=("warm64",), window=1000)
    plain = np.array([r["plain_its"] for r in rows], dtype=float)
    warm = np.array([r["warm64_its"] for r in rows], dtype=float)
    print("iterations to Cd within 1%: plain", plain.tolist(), "warm", warm.tolist())
    assert np.all(np.isfinite(plain)) and np.all(np.isfinite(warm))
    # every held-out case converges sooner from the prediction, the median
    # case at least 1.5x sooner; both runs end at the same Cd
    assert np.all(warm < plain)
    assert np.median(plain / warm) >= 1.5
    assert max(r["warm64_cd_err"] for r in rows) < 1e-3
