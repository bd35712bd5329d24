"""Regenerate tests/golden/oracle_golden.json.

The fixture pins the CPU oracle: for each case it holds the Monitor series
and SHA-256 digests of f, fb, p, u after a fixed number of iterations, as
computed by the array-oriented numpy restatement in numpy_reference.py
(independent of oracle/lbm_oracle.c). Run from the repository root:

    python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from numpy_reference import NumpyLBM  # noqa: E402

CASES = {
    # name: (dim, nx, ny, nz, input.in line 2, line 3, r_vec seed, iterations, interv)
    "cylinder_2d_40x20": (2, 40, 20, 0, (0.3, 0.3, 20.0), (1.75, 1.0, 1.1), 5, 30, 4),
    "cylinder_2d_64x32": (2, 64, 32, 0, (0.25, 0.25, 20.0), (1.8, 1.0, 1.0), 12345, 25, 5),
    "sphere_3d_20x10x12": (3, 20, 10, 12, (0.3, 0.3, 20.0), (1.75, 1.0, 1.1), 5, 12, 4),
}


def r_vec(seed):
    """splitmix64 -> 53-bit uniforms, the seeded InitUP draws of the host API."""
    out, x = [], seed
    m = (1 << 64) - 1
    for _ in range(100):
        x = (x + 0x9E3779B97F4A7C15) & m
        z = x
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & m
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & m
        z ^= z >> 31
        out.append((z >> 11) * 2.0 ** -53)
    return np.array(out)


def digest(a):
    a = np.ascontiguousarray(a, dtype=np.float64).ravel().copy()
    a[np.isnan(a)] = np.nan  # one NaN pattern
    a[a == 0] = 0.0          # one zero
    return hashlib.sha256(a.tobytes()).hexdigest()


def make():
    out = {}
    for name, (dim, nx, ny, nz, (L, xp, re), (ome, dt, rho0), seed, n, iv) in CASES.items():
        m = NumpyLBM(dim, nx, ny, nz, L, xp, re, ome, dt, rho0)
        m.init_up(r_vec(seed))
        m.init_pdf()
        log = m.run(0, n, iv)
        out[name] = {"dim": dim, "n": [nx, ny, nz], "line2": [L, xp, re], "line3": [ome, dt, rho0],
                     "seed": seed, "iterations": n, "interv": iv,
                     "r_vec_head": r_vec(seed)[:4].tolist(),
                     "monitor": [float(v) for v in log],
                     "sha256": {"f": digest(m.f), "fb": digest(m.fb), "p": digest(m.p),
                                "u": digest(m.u)}}
    return out


if __name__ == "__main__":
    with open(os.path.join(HERE, "oracle_golden.json"), "w") as fh:
        json.dump(make(), fh, indent=1)
    print("wrote", os.path.join(HERE, "oracle_golden.json"))
