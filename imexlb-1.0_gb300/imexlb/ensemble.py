"""Ensemble of independent D2Q9 cylinder flows advanced in lockstep on one GPU.

The data generator of the learned warm start: each case is the reference's
2D flow past a cylinder (reference geometry, boundary program and BGK
update) with its own lattice size, diameter, Reynolds number and a small
vertical offset of the cylinder (an extension of the reference geometry).
All cases advance together through imexlb_batch_* with reduced-precision
storage; every `snapshot_every` iterations each active case is sampled on a
fixed 256 x 128 grid (fluid fraction, p, ux, uy).

    python -m imexlb.ensemble --cases 256 --out ensemble.npz
"""
import argparse
import time

import numpy as np

from . import BATCH_LOCKSTEP, BATCH_PERSISTENT, FP16, FP32, BF16, Batch, Setup, Solver, make_config

U_IN = 0.05


def draw_cases(n=256, seed=0, nx_range=(256, 1024), d_range=(16.0, 48.0), re_range=(40.0, 200.0),
               yoff=2.0):
    """Seeded case table: nx uniform over multiples of 32, ny = nx/2,
    diameter, Reynolds number and y offset uniform; centre at x = nx/4."""
    rng = np.random.default_rng(seed)
    lo, hi = nx_range[0] // 32, nx_range[1] // 32
    out = []
    for _ in range(n):
        nx = int(rng.integers(lo, hi + 1)) * 32
        out.append(dict(nx=nx, ny=nx // 2, D=float(rng.uniform(*d_range)),
                        re=float(rng.uniform(*re_range)), yoff=float(rng.uniform(-yoff, yoff)),
                        steps=8 * nx))
    return out


def case_config(c, u_in=U_IN):
    """input.in values of a case: L = D/nx, Xpos = 1/4, Re, ome from
    nu = u_in*D/Re (so DataInput's uu = Re*nu/L equals u_in)."""
    nu = u_in * c["D"] / c["re"]
    ome = 1.0 / (3.0 * nu + 0.5)
    return make_config(2, c["nx"], c["ny"], charlength=c["D"] / c["nx"], xpos=0.25, re=c["re"],
                       ome=ome, yoff=c["yoff"])


def make_solver(c, precision=FP32, device=0, init="rest"):
    """Solver of one case after its first iteration. init='rest': p = u = 0
    (the inlet Dirichlet profile acts from the first PostProcessing);
    init='reference': the reference's InitUP."""
    cfg = case_config(c)
    # SetGeometry on the device; the initial state is computed there too
    st = Setup(cfg, device=device, state=False)
    s = Solver(cfg, precision=precision, device=device)
    s.set_geometry(st)
    # no full-array uploads
    s.init_state(None if init == "rest" else st.r_vec)
    s.init_pdf()
    s.step(0, 1)
    return s, cfg


def run(cases, precision=FP32, snapshot_every=500, W=256, H=128, tune=True, device=0,
        keep_snapshots=True, mean_last=0.0, log=print, mode=BATCH_LOCKSTEP):
    """Advance every case to its iteration budget in one batch (mode:
    BATCH_LOCKSTEP, one graph-replayed launch pair per iteration with an
    autotuned shape when `tune`, the faster on GB300; or BATCH_PERSISTENT, one
    cooperative launch per call). Returns a dict
    with per-case snapshots (list of (iteration, float16 array (4,H,W))), the
    final sample, the time mean of the samples taken in the last `mean_last`
    fraction of each case's budget (when > 0), and timing: node updates, GPU
    seconds, MLUPS."""
    t0 = time.perf_counter()
    solvers = []
    for c in cases:
        s, _ = make_solver(c, precision, device)
        solvers.append(s)
    t_setup = time.perf_counter() - t0
    done = np.ones(len(cases), dtype=np.int64)  # first iteration taken
    budget = np.array([c["steps"] for c in cases], dtype=np.int64)
    nodes = np.array([(c["nx"] + 1) * (c["ny"] + 1) for c in cases], dtype=np.int64)
    snaps = [[] for _ in cases]
    mean_sum = [None] * len(cases)
    mean_cnt = np.zeros(len(cases), dtype=np.int64)
    shape = None
    gpu_s = 0.0
    updates = int((nodes * 1).sum())
    with Batch(solvers) as b:
        b.set_mode(mode)
        if tune and mode == BATCH_LOCKSTEP:
            tt = time.perf_counter()
            shape = b.tune(trial=4)
            gpu_s += time.perf_counter() - tt
            done += 4 * 6
            updates += int((nodes * 4 * 6).sum())
        while np.any(done < budget):
            next_stop = (done // snapshot_every + 1) * snapshot_every
            steps = np.minimum(next_stop, budget) - done
            steps[done >= budget] = 0
            tt = time.perf_counter()
            b.step(steps=steps.astype(np.int32))
            gpu_s += time.perf_counter() - tt
            updates += int((nodes * steps).sum())
            done += steps
            for i in np.flatnonzero((steps > 0) & ((done % snapshot_every == 0) | (done >= budget))):
                if not keep_snapshots and not (mean_last > 0 and done[i] >= (1 - mean_last) * budget[i]):
                    continue
                smp = solvers[i].sample(W, H)
                if keep_snapshots:
                    snaps[i].append((int(done[i]), smp.astype(np.float16)))
                if mean_last > 0 and done[i] >= (1 - mean_last) * budget[i]:
                    mean_sum[i] = smp.astype(np.float64) if mean_sum[i] is None else mean_sum[i] + smp
                    mean_cnt[i] += 1
    final = [s.sample(W, H) for s in solvers]
    for s in solvers:
        s.close()
    mean = [m / c if m is not None else f for m, c, f in zip(mean_sum, mean_cnt, final)]
    res = dict(snapshots=snaps, final=final, mean=mean, node_updates=updates, gpu_seconds=gpu_s,
               mlups=updates / gpu_s / 1e6, setup_seconds=t_setup, shape=shape)
    log("ensemble: %d cases, %.3g node updates in %.2f s (%.0f MLUPS incl. snapshots), setup %.1f s, shape %s"
        % (len(cases), updates, gpu_s, res["mlups"], t_setup, shape))
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--cases", type=int, default=256)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--precision", default="fp32", choices=["fp32", "bf16", "fp16"])
    ap.add_argument("--snapshot-every", type=int, default=500)
    ap.add_argument("--mode", default="lockstep", choices=["lockstep", "persistent"])
    ap.add_argument("--out", default="")
    a = ap.parse_args()
    prec = {"fp32": FP32, "bf16": BF16, "fp16": FP16}[a.precision]
    cases = draw_cases(a.cases, a.seed)
    res = run(cases, prec, a.snapshot_every,
              mode=BATCH_PERSISTENT if a.mode == "persistent" else BATCH_LOCKSTEP)
    if a.out:
        np.savez_compressed(
            a.out,
            mask=np.stack([f[0] for f in res["final"]]).astype(np.float16),
            re=np.array([c["re"] for c in cases]), D=np.array([c["D"] for c in cases]),
            nx=np.array([c["nx"] for c in cases]),
            final=np.stack([f[1:] for f in res["final"]]).astype(np.float16))


if __name__ == "__main__":
    main()
