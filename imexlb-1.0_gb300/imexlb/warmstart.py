"""Learned warm start of the D2Q9 cylinder flow and its evaluation.

Pipeline: an ensemble of cylinder flows (imexlb.ensemble) provides training
pairs (fluid fraction + Re on a 256 x 128 grid -> sampled p, ux, uy); the
network (imexlb.neural) is trained with the library's tensor-core kernels;
for a held-out case the prediction is interpolated to the lattice nodes and
becomes the initial p, u of the solver (f = feq via InitPDF).

Evaluation, per held-out case (1024 x 512 lattice): the plain run starts from
rest in FP64; the warm runs start from the prediction in FP16 (and in FP64,
to separate the network's effect from the precision's). Drag and lift come
from the momentum-exchange force every `every` iterations:
Cd = 2 Fx / (rho0 U^2 D), Cl = 2 Fy / (rho0 U^2 D). The plain run's last
`tail` fraction gives the converged mean Cd and the Strouhal number
St = f D / U (f the dominant frequency of Cl, from a Hann-windowed FFT); a
run "has converged" at the first checkpoint after which its windowed Cd (and
St) stay within 1 % of those values until the end. Time to converge = that iteration count times
the run's measured wall time per iteration.
"""
import time

import numpy as np

from . import FP16, FP64, Setup, Solver, neural
from .ensemble import U_IN, case_config, draw_cases

W_GRID, H_GRID = 256, 128


def fluid_fraction(st, cfg, W=W_GRID, H=H_GRID):
    """Bilinear sample of the fluid indicator at the W x H pixel centres
    (the same rule as imexlb_sample's first channel)."""
    L0, L1 = cfg.nx + 1, cfg.ny + 1
    dy = cfg.dy
    geo = st.geo.reshape(-1, dy)[3:3 + L1, 3:3 + L0].astype(np.float32)
    X = np.clip((np.arange(W) + 0.5) * L0 / W - 0.5, 0, L0 - 1)
    Y = np.clip((np.arange(H) + 0.5) * L1 / H - 0.5, 0, L1 - 1)
    x0 = np.minimum(X.astype(int), L0 - 2)
    y0 = np.minimum(Y.astype(int), L1 - 2)
    fx, fy = (X - x0)[None, :], (Y - y0)[:, None]
    g = lambda yy, xx: geo[yy[:, None], xx[None, :]]
    return ((1 - fy) * ((1 - fx) * g(y0, x0) + fx * g(y0, x0 + 1)) +
            fy * ((1 - fx) * g(y0 + 1, x0) + fx * g(y0 + 1, x0 + 1)))


def to_nodes(field, cfg):
    """Interpolate a (H, W) pixel-centre field to the (ny+1, nx+1) nodes."""
    H, W = field.shape
    L0, L1 = cfg.nx + 1, cfg.ny + 1
    X = np.clip((np.arange(L0) + 0.5) * W / L0 - 0.5, 0, W - 1)
    Y = np.clip((np.arange(L1) + 0.5) * H / L1 - 0.5, 0, H - 1)
    x0 = np.minimum(X.astype(int), W - 2)
    y0 = np.minimum(Y.astype(int), H - 2)
    fx, fy = (X - x0)[None, :], (Y - y0)[:, None]
    g = lambda yy, xx: field[yy[:, None], xx[None, :]]
    return ((1 - fy) * ((1 - fx) * g(y0, x0) + fx * g(y0, x0 + 1)) +
            fy * ((1 - fx) * g(y0 + 1, x0) + fx * g(y0 + 1, x0 + 1)))


def training_set(res, cases):
    """(fluid fraction, Re, fields) from an ensemble result: the time-mean
    samples when present, else the final ones."""
    fin = np.stack(res.get("mean") or res["final"])
    frac = fin[:, 0].astype(np.float32)
    fields = fin[:, 1:4].astype(np.float32)
    re = np.array([c["re"] for c in cases], dtype=np.float32)
    return frac, re, fields


def _solver(c, precision, p=None, u=None):
    cfg = case_config(c)
    st = Setup(cfg)
    st.p[:] = 0.0
    st.u[:] = 0.0
    if p is not None:
        st.p[:] = p
        st.u[:] = u
    s = Solver(cfg, precision=precision)
    s.set_geometry(st)
    s.upload(st.f, st.fb, st.p, st.u)
    s.init_pdf()
    return s, cfg, st


def warm_fields(net, c):
    """Predicted p, u (reference layout) for a case."""
    cfg = case_config(c)
    st = Setup(cfg)
    frac = fluid_fraction(st, cfg)[None]
    pred = neural.predict(net, frac, np.array([c["re"]]))[0]
    dy = cfg.dy
    n = cfg.array_size
    p = np.zeros(n)
    u = np.zeros(2 * n)
    L0, L1 = cfg.nx + 1, cfg.ny + 1
    ids = (np.arange(L1)[:, None] + 3) * dy + (np.arange(L0)[None, :] + 3)
    fluid = st.geo[ids] == 1
    P, UX, UY = (to_nodes(pred[k], cfg) for k in range(3))
    sel = ids[fluid]
    p[sel] = P[fluid]
    u[2 * sel] = UX[fluid]
    u[2 * sel + 1] = UY[fluid]
    return p, u


def run_forces(s, cfg, c, steps, every, chunk=2000):
    """Advance and record Cd, Cl every `every` iterations; returns
    (iterations, Cd, Cl, seconds per iteration)."""
    Fs = []
    t0 = time.perf_counter()
    it = 0
    while it < steps:
        k = min(chunk, steps - it)
        _, F = s.step_observed(it, k, 0, every)
        Fs.append(F)
        it += k
    dt = (time.perf_counter() - t0) / steps
    F = np.concatenate(Fs)
    q = 2.0 / (cfg.rho0 * cfg.uu ** 2 * c["D"])
    its = np.arange(0, steps, every) + 1
    return its, F[:, 0] * q, F[:, 1] * q, dt


def strouhal(cl, every, D, U):
    """St = f D / U with f the dominant frequency of Cl (Hann-windowed FFT,
    parabolic refinement of the peak); NaN when Cl does not oscillate."""
    x = np.asarray(cl, dtype=np.float64)
    x = x - x.mean()
    if len(x) < 16 or np.std(x) < 1e-4:
        return float("nan")
    n = len(x)
    spec = np.abs(np.fft.rfft(x * np.hanning(n), n=4 * n))
    spec[0] = 0.0
    k = int(np.argmax(spec))
    if k <= 0 or k >= len(spec) - 1:
        return float("nan")
    a, b, c = np.log(spec[k - 1] + 1e-300), np.log(spec[k] + 1e-300), np.log(spec[k + 1] + 1e-300)
    dk = 0.5 * (a - c) / (a - 2 * b + c) if (a - 2 * b + c) != 0 else 0.0
    freq = (k + dk) / (4 * n * every)  # cycles per iteration
    # fewer than two periods in the window: no reliable frequency
    if freq * n * every < 2.0:
        return float("nan")
    return freq * D / U


def converged_values(its, cd, cl, every, D, U, tail=0.25):
    n = len(cd)
    sl = slice(int(n * (1 - tail)), n)
    return float(np.mean(cd[sl])), strouhal(cl[sl], every, D, U)


def time_to_within(its, cd, cl, every, D, U, cd_ref, st_ref, window, tol=0.01):
    """First iteration after which the trailing-window mean Cd (and the
    window's St when the reference has one) stay within tol of the reference
    at every later checkpoint until the end; None if never."""
    n = len(cd)
    w = max(8, window // every)
    stride = max(1, w // 8)
    checks = list(range(w, n + 1, stride))
    if not checks or checks[-1] != n:
        checks.append(n)
    ok = []
    for i in checks:
        good = abs(np.mean(cd[i - w:i]) - cd_ref) <= tol * abs(cd_ref)
        if good and np.isfinite(st_ref):
            st = strouhal(cl[i - w:i], every, D, U)
            good = bool(np.isfinite(st) and abs(st - st_ref) <= tol * st_ref)
        ok.append(good)
    ok = np.array(ok)
    bad = np.flatnonzero(~ok)
    j = 0 if len(bad) == 0 else bad[-1] + 1
    if j >= len(checks):
        return None
    return int(its[checks[j] - 1])


WARM_KINDS = {"warm16": FP16, "warm64": FP64}


def train_network(ncases=256, nx_range=(256, 1024), nx_iters=60, mean_last=0.33, train_steps=2000,
                  batch=16, seed=0, d_range=(16.0, 48.0), re_range=(40.0, 200.0)):
    """The training pipeline: an ensemble of cylinder flows (nx_iters * nx
    iterations per case, the time mean of the last `mean_last` of each run
    sampled on the 256 x 128 grid), then Adam on the network. Returns the
    network and timings."""
    import torch
    from . import FP32, ensemble
    cases = draw_cases(ncases, seed=seed, nx_range=nx_range, d_range=d_range, re_range=re_range)
    for c in cases:
        c["steps"] = nx_iters * c["nx"]
    t0 = time.perf_counter()
    res = ensemble.run(cases, FP32, keep_snapshots=False, mean_last=mean_last, log=lambda *x: None)
    t1 = time.perf_counter()
    frac, re, fields = training_set(res, cases)
    net = neural.Net(seed=seed)
    hist = neural.train(net, frac, re, fields, steps=train_steps, batch=batch)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    return net, {"ensemble_s": t1 - t0, "ensemble_mlups": res["mlups"], "train_s": t2 - t1,
                 "loss_first": hist[0][1], "loss_last": hist[-1][1]}


def evaluate(net, seeds, steps=60000, every=20, nx=1024, log=print, d_range=(16.0, 48.0),
             re_range=(40.0, 200.0), warm=("warm16", "warm64"), window=None):
    """Per held-out seed: the plain FP64 run from rest (the arbiter: its last
    quarter gives the converged Cd and St) and the warm-started runs `warm`
    (keys of WARM_KINDS); iterations and wall time per iteration of each until
    its Cd / St stay within 1 % of the plain run's converged values."""
    rows = []
    for seed in seeds:
        c = draw_cases(1, seed=seed, nx_range=(nx, nx), d_range=d_range, re_range=re_range)[0]
        c["steps"] = steps
        # about 5 shedding periods unless given
        win = window if window is not None else int(5 * c["D"] / (0.2 * U_IN))
        out = {"seed": seed, "Re": c["re"], "D": c["D"]}
        s, cfg, _ = _solver(c, FP64)
        its, cd, cl, dtp = run_forces(s, cfg, c, steps, every)
        s.close()
        cd_ref, st_ref = converged_values(its, cd, cl, every, c["D"], cfg.uu)
        out.update(cd_ref=cd_ref, st_ref=st_ref, plain_ms_per_it=dtp * 1e3)
        t_plain = time_to_within(its, cd, cl, every, c["D"], cfg.uu, cd_ref, st_ref, win)
        out["plain_its"] = t_plain
        p, u = warm_fields(net, c)
        for name in warm:
            s, cfg, _ = _solver(c, WARM_KINDS[name], p, u)
            its_w, cd_w, cl_w, dtw = run_forces(s, cfg, c, steps, every)
            s.close()
            out[name + "_its"] = time_to_within(its_w, cd_w, cl_w, every, c["D"], cfg.uu, cd_ref,
                                                st_ref, win)
            out[name + "_ms_per_it"] = dtw * 1e3
            out[name + "_cd_err"] = abs(np.mean(cd_w[-len(cd_w) // 3:]) - cd_ref) / abs(cd_ref)
        rows.append(out)
        log(out)
    return rows


def main():
    """Ensemble -> training -> evaluation on held-out seeds; prints JSON lines."""
    import argparse
    import json
    import torch
    from . import FP32
    from . import ensemble
    ap = argparse.ArgumentParser()
    ap.add_argument("--cases", type=int, default=256)
    ap.add_argument("--train-nx-iters", type=int, default=60,
                    help="ensemble iterations per case as a multiple of nx (8 = the data-generation run)")
    ap.add_argument("--mean-last", type=float, default=0.33)
    ap.add_argument("--train-steps", type=int, default=2000)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--seeds", type=int, default=32)
    ap.add_argument("--first-seed", type=int, default=1000)
    ap.add_argument("--steps", type=int, default=100000)
    ap.add_argument("--every", type=int, default=20)
    ap.add_argument("--nx", type=int, default=1024)
    a = ap.parse_args()
    emit = lambda d: print(json.dumps(d), flush=True)
    cases = ensemble.draw_cases(a.cases, seed=0)
    for c in cases:
        c["steps"] = a.train_nx_iters * c["nx"]
    res = ensemble.run(cases, FP32, keep_snapshots=False, mean_last=a.mean_last, log=lambda *x: None)
    emit({"stage": "ensemble", "cases": a.cases, "mlups": res["mlups"],
          "gpu_seconds": res["gpu_seconds"]})
    frac, re, fields = training_set(res, cases)
    net = neural.Net(seed=0)
    t0 = time.perf_counter()
    hist = neural.train(net, frac, re, fields, steps=a.train_steps, batch=a.batch)
    torch.cuda.synchronize()
    emit({"stage": "train", "steps": a.train_steps, "seconds": time.perf_counter() - t0,
          "loss_first": hist[0][1], "loss_last": hist[-1][1]})
    rows = evaluate(net, range(a.first_seed, a.first_seed + a.seeds), steps=a.steps, every=a.every,
                    nx=a.nx, log=lambda r: emit(dict(stage="case", **r)))
    emit({"stage": "summary", **summarize(rows)})


def summarize(rows, warm=("warm16", "warm64")):
    """Speed-ups of the warm starts over the plain run (wall time to within 1 %)."""
    out = {"cases": len(rows)}
    for name in warm:
        sp, conv = [], 0
        for r in rows:
            if r["plain_its"] is None or r[name + "_its"] is None:
                continue
            conv += 1
            tp = r["plain_its"] * r["plain_ms_per_it"]
            tw = max(r[name + "_its"], 1) * r[name + "_ms_per_it"]
            sp.append(tp / tw)
        out[name] = {"converged": conv, "median_speedup": float(np.median(sp)) if sp else None,
                     "mean_speedup": float(np.mean(sp)) if sp else None,
                     "frac_ge_2x": float(np.mean(np.array(sp) >= 2.0)) if sp else None,
                     "median_cd_err": float(np.median([r[name + "_cd_err"] for r in rows]))}
    return out


if __name__ == "__main__":
    main()
