"""Reduced-precision storage against the FP64 path on one workload.

Runs the same case (reference geometry, InitUP with seeded draws, InitPDF)
once per storage kind for the same number of iterations, recording the
momentum-exchange drag every `every` iterations, and reports per kind: mean
Cd over the last third, its relative difference to FP64, the relative L2
error of the velocity field over fluid nodes, the drift of the fluid mass
sum over the run relative to FP64's, and MLUPS. The FP64 run is the
reference-rounding path (bit-identical to the CPU oracle); fp64fast is the
minimal-operation FP64 update with fused multiply-adds.

    python -m imexlb.precision_study --nx 512 --ny 256 --nz 256 --steps 5000
"""
import argparse
import json
import time

import numpy as np

from . import BF16, FP16, FP32, FP64, FP64_FAST, Setup, Solver, make_config

KINDS = {"fp64": FP64, "fp64fast": FP64_FAST, "fp32": FP32, "bf16": BF16, "fp16": FP16}


def run_kind(cfg, st, kind, steps, every):
    s = Solver(cfg, precision=KINDS[kind])
    s.set_geometry(st)
    s.upload(st.f, st.fb, st.p, st.u)
    s.init_pdf()
    _, m0 = s.observe()
    t0 = time.perf_counter()
    _, F = s.step_observed(0, steps, 0, every)
    dt = time.perf_counter() - t0
    _, m1 = s.observe()
    _, _, _, u = s.download(f=False, fb=False, p=False)
    s.close()
    return F, u, m0, m1, dt


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--dim", type=int, default=3)
    ap.add_argument("--nx", type=int, default=512)
    ap.add_argument("--ny", type=int, default=256)
    ap.add_argument("--nz", type=int, default=256)
    ap.add_argument("--D", type=float, default=48.0)
    ap.add_argument("--re", type=float, default=200.0)
    ap.add_argument("--u", type=float, default=0.04)
    ap.add_argument("--steps", type=int, default=5000)
    ap.add_argument("--every", type=int, default=50)
    ap.add_argument("--kinds", default="fp64,fp64fast,fp32,fp16,bf16")
    a = ap.parse_args()
    nu = a.u * a.D / a.re
    cfg = make_config(a.dim, a.nx, a.ny, a.nz, charlength=a.D / a.nx, xpos=0.25, re=a.re,
                      ome=2.0 / (1.0 + 6.0 * nu))
    st = Setup(cfg, seed=12345)
    nodes = cfg.nodes
    area = np.pi * a.D ** 2 / 4 if a.dim == 3 else a.D
    q = 2.0 / (cfg.rho0 * cfg.uu ** 2 * area)
    fid = st.fluid_id
    ref = None
    for kind in a.kinds.split(","):
        F, u, m0, m1, dt = run_kind(cfg, st, kind, a.steps, a.every)
        cd = F[:, 0] * q
        cd_mean = float(np.mean(cd[-max(1, len(cd) // 3):]))
        uf = u.reshape(-1, a.dim)[fid]
        row = {"kind": kind, "steps": a.steps, "nodes": nodes, "mlups": nodes * a.steps / dt / 1e6,
               "cd": cd_mean, "mass_drift": (m1 - m0)}
        if ref is None:
            ref = (cd_mean, uf, m1 - m0, row["mlups"])
        else:
            row["cd_rel_err"] = abs(cd_mean - ref[0]) / abs(ref[0])
            row["u_rel_l2"] = float(np.linalg.norm(uf - ref[1]) / np.linalg.norm(ref[1]))
            row["mass_drift_minus_fp64"] = (m1 - m0) - ref[2]
            row["speedup_vs_fp64"] = row["mlups"] / ref[3]
        print(json.dumps(row), flush=True)


if __name__ == "__main__":
    main()
