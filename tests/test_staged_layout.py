"""CPU: the copies of the staged step kernel stay inside their buffers.

The staged kernel of the 2-byte kinds (kernels_lp.cu, k_step_staged, with
the copy plan of staged.cuh) copies, for each tile of TILE = 1024 cells from
id_lo, every direction's pulled run from the 16-byte boundary below its first
element, TILE * sizeof(T) + 16 bytes, and the tile's mask bytes from the
16-byte boundary below the tile, TILE + 16 bytes. The launch takes the staged
kernel only where the trailing ghost layers cover that (N - id_hi >= TILE +
16 + dy + dz); this test restates the copy extents with the lattice layout
of the library's host setup and checks, for every tile of every lattice the
tests and the benchmark run, that each copy lies inside the population buffer (Q N elements at a 256-byte aligned base) and inside
the mask (N bytes), that the run's element TILE (the inlet pull one cell on)
lies inside its copy, and that every run's position in a stage fits the
32-bit plan entry.
"""
import numpy as np
import pytest

GHOST = 3
# (element bytes, cells per tile) of the staged kernel: BF16 / FP16
KINDS = [(2, 1024)]


def layout(cfg, e):
    dim = cfg.dim
    L = [cfg.local_length[k] if k < dim else 1 for k in range(3)]
    dy, dz = cfg.dy, (cfg.dz if dim == 3 else 0)
    N = dy * (L[1] + 2 * GHOST) * ((L[2] + 2 * GHOST) if dim == 3 else 1)
    id_lo = GHOST + dy * GHOST + dz * GHOST
    id_hi = (L[0] + GHOST - 1) + dy * (L[1] + GHOST - 1) + (dz * (L[2] + GHOST - 1) if dim == 3 else 0) + 1
    ev = e.reshape(-1, dim)
    off = ev[:, 0] + ev[:, 1] * dy + (ev[:, 2] * dz if dim == 3 else 0)
    return N, id_lo, id_hi, dy, dz, off.astype(np.int64)


def fits(N, id_hi, dy, dz, tile):
    return N - id_hi >= tile + 16 + dy + dz


def cases():
    from parity_util import CASES
    out = [(n, c[0], c[1], c[2], c[3]) for n, c in CASES.items()]
    import bench
    for n, w in bench.WORKLOADS.items():
        out.append((n, w["dim"], w["nx"], w["ny"], w["nz"]))
    out += [("2d_128x64", 2, 128, 64, 0), ("2d_250x40", 2, 250, 40, 0), ("3d_17x9x5", 3, 17, 9, 5)]
    return out


@pytest.mark.parametrize("case", cases(), ids=lambda c: c[0])
@pytest.mark.parametrize("esz,TILE", KINDS)
def test_staged_copies_stay_in_their_buffers(case, esz, TILE):
    import imexlb as im
    name, dim, nx, ny, nz = case
    cfg = im.make_config(dim, nx, ny, nz)
    t, e = im.lattice(dim)
    Q = t.size
    N, id_lo, id_hi, dy, dz, off = layout(cfg, e)
    if not fits(N, id_hi, dy, dz, TILE):
        # the launch keeps the register kernel (ghost layers thinner than a
        # tile's copies): small lattices only
        assert N < 2_000_000, name
        return
    run = TILE * esz + 16
    ntiles = (id_hi - id_lo + TILE - 1) // TILE
    c0 = id_lo + TILE * np.arange(ntiles, dtype=np.int64)
    for base in (0, 256 * 7):  # any 256-byte aligned allocation
        for i in range(Q):
            first = base + esz * (i * N - off[i] + c0)  # byte address of the run's element 0
            a0 = first & ~np.int64(15)
            assert np.all(a0 >= base) and np.all(a0 + run <= base + esz * Q * N), (name, i)
            # element TILE (inlet pull of the tile's last cell) inside the copy
            assert np.all(first + esz * (TILE + 1) <= a0 + run)
            pos = i * run + int((first[0] - a0[0]))
            assert np.all(first - a0 == first[0] - a0[0])  # the same for every tile
            assert pos < 2 ** 32
        m0 = (base + c0) & ~np.int64(15)
        assert np.all(m0 >= base) and np.all(m0 + TILE + 16 <= base + N)
        assert np.all(base + c0 + TILE <= m0 + TILE + 16)
    # the tile cells past id_hi are masked out in the kernel; the boundary
    # group indices (id - id_lo) / 64 fit 32 bits
    assert (id_hi - id_lo) // 64 < 2 ** 32


@pytest.mark.parametrize("name", ["3d_32x16x16", "3d_24x12x14_rho", "sphere_d3q27_128x64x64",
                                  "sphere_d3q27_256x128x128", "sphere_d3q27_512x256x256"])
@pytest.mark.parametrize("esz,TILE", KINDS)
def test_staged_kernel_runs_on_the_tested_lattices(name, esz, TILE):
    """The GPU tests of the staged kernel compare it with the register kernel
    on these lattices: each must take the staged kernel."""
    import imexlb as im
    c = {n: (dim, nx, ny, nz) for n, dim, nx, ny, nz in cases()}[name]
    cfg = im.make_config(*c)
    _, e = im.lattice(c[0])
    N, _, id_hi, dy, dz, _ = layout(cfg, e)
    assert fits(N, id_hi, dy, dz, TILE), name
