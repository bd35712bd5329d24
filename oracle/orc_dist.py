"""The reference's multi-rank program with one OS process per MPI rank.

TEST INFRASTRUCTURE ONLY (the checker of the rank-group path): the oracle's
per-rank routines (lbm_oracle.c) driven as cart_mpi.f90 drives them, with
PassInt / PassF as point-to-point torch.distributed messages of the ghost
cells each rank needs from each other rank (every rank derives the whole
exchange plan from the decomposition, so no handshake is needed) and Monitor
as an all-reduce MAX (lbm.f90:209-220). Run under any backend; the tests use
gloo on CPU.
"""
import ctypes as C

import numpy as np

from . import orc

G = 3


def _rank_coords(r, nps):
    if len(nps) == 2:
        return (r // nps[1], r % nps[1])
    return (r // (nps[1] * nps[2]), (r // nps[2]) % nps[1], r % nps[2])


def _rank_of(c, nps):
    if len(nps) == 2:
        return c[0] * nps[1] + c[1]
    return (c[0] * nps[1] + c[1]) * nps[2] + c[2]


class Layout:
    """Decomposition of the global lattice over nprocs ranks."""

    def __init__(self, dim, gl, nprocs):
        self.dim, self.gl, self.nprocs = dim, tuple(gl), nprocs
        self.nps = orc.decompose(dim, gl, nprocs)
        self.boxes = [orc.local_box(dim, gl, self.nps, _rank_coords(r, self.nps)) for r in range(nprocs)]

    def strides(self, r):
        L, _ = self.boxes[r]
        dy = L[0] + 2 * G
        dz = dy * (L[1] + 2 * G) if self.dim == 3 else 0
        return dy, dz

    def ghost_sources(self, a):
        """For rank a: (ghost cells of a, owner rank, owner cell) of PassF."""
        L, st = self.boxes[a]
        dim = self.dim
        pads = [L[d] + 2 * G for d in range(dim)]
        grids = np.meshgrid(*[np.arange(p) for p in pads], indexing="ij")
        P = [g.ravel() for g in grids]  # X, Y[, Z] padded coordinates
        ghost = np.zeros(P[0].size, dtype=bool)
        for d in range(dim):
            ghost |= (P[d] < G) | (P[d] >= L[d] + G)
        P = [p[ghost] for p in P]
        dy, dz = self.strides(a)
        dst = P[0] + dy * P[1] + (dz * P[2] if dim == 3 else 0)
        owner_c = []
        loc = []
        for d in range(dim):
            gx = (P[d] - G + st[d]) % self.gl[d]
            lens = [self.gl[d] // self.nps[d] + (1 if c < self.gl[d] % self.nps[d] else 0)
                    for c in range(self.nps[d])]
            starts = np.cumsum([0] + lens[:-1])
            c = np.searchsorted(starts, gx, side="right") - 1
            owner_c.append(c)
            loc.append(gx - starts[c] + G)
        owner = np.array([_rank_of(tuple(int(owner_c[d][i]) for d in range(dim)), self.nps)
                          for i in range(dst.size)], dtype=np.int64)
        src = np.zeros(dst.size, dtype=np.int64)
        for b in np.unique(owner):
            m = owner == b
            bdy, bdz = self.strides(int(b))
            src[m] = loc[0][m] + bdy * loc[1][m] + (bdz * loc[2][m] if dim == 3 else 0)
        return dst.astype(np.int64), owner, src


class DistRank:
    """This process's rank of the reference run."""

    def __init__(self, inp, dist, nthreads=1, allow_geom_error=False):
        import torch
        self.torch = torch
        self.dist = dist
        self.rank, self.world = dist.get_rank(), dist.get_world_size()
        gl = (inp.nx + 1, inp.ny + 1) + ((inp.nz + 1,) if inp.dim == 3 else ())
        self.lay = Layout(inp.dim, gl, self.world)
        L, st = self.lay.boxes[self.rank]
        pad = lambda v, fill: (C.c_int * 3)(*(list(v) + [fill] * (3 - len(v))))
        self.s = orc.OrcState()
        rc = orc.lib().orc_setup_rank(C.byref(self.s), C.byref(inp), pad(L, 1), pad(st, 0))
        if rc != 0:
            raise ValueError("rank setup failed (rc=%d)" % rc)
        self.o = orc.Oracle(None, nthreads, _state=self.s, _owner=self)
        # exchange plan: what this rank receives from each rank, and sends
        self.recv = {}
        dst, owner, src = self.lay.ghost_sources(self.rank)
        for b in np.unique(owner):
            m = owner == b
            self.recv[int(b)] = (dst[m], src[m])
        self.send = {}
        for a in range(self.world):
            if a == self.rank:
                continue
            d, ow, sr = self.lay.ghost_sources(a)
            m = ow == self.rank
            if m.any():
                self.send[a] = sr[m]
        self._exchange(self.o.geo, 1)  # PassInt(geo)
        rc = orc.lib().orc_obstacle_scan(C.byref(self.s))
        if rc != 0 and not allow_geom_error:
            raise ValueError("obstacle probe left the geo array")

    def _exchange(self, arr, width):
        """PassF / PassInt: ghost cells receive the owners' interior cells."""
        torch = self.torch
        a2 = arr.reshape(-1, width)
        reqs = []
        bufs = {}
        for b, (dst, src) in sorted(self.recv.items()):
            if b == self.rank:
                continue
            bufs[b] = torch.empty(dst.size * width, dtype=torch.float64)
            reqs.append(self.dist.irecv(bufs[b], src=b))
        for b, src in sorted(self.send.items()):
            out = torch.from_numpy(np.ascontiguousarray(a2[src], dtype=np.float64).ravel())
            reqs.append(self.dist.isend(out, dst=b))
        if self.rank in self.recv:  # periodic images of this rank's own cells
            dst, src = self.recv[self.rank]
            a2[dst] = a2[src]
        for r in reqs:
            r.wait()
        for b, buf in bufs.items():
            dst, _ = self.recv[b]
            a2[dst] = buf.numpy().reshape(-1, width).astype(a2.dtype)

    def init_up(self, rv):
        self.o.init_up(rv)

    def init_pdf(self):
        self.o.init_pdf()

    def monitor(self):
        t = self.torch.tensor([self.o.monitor()], dtype=self.torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t[0])

    def run(self, iter0, nsteps, interv):
        log = []
        for it in range(iter0, iter0 + nsteps):
            if interv > 0 and it % interv == 0:
                log.append(self.monitor())
            self.o.collision()
            self._exchange(self.o.fb, self.s.nq)  # PassF
            self.o.bc_copies()
            self.o.propagation()
            self.o.post_processing()
        return np.array(log)

    def close(self):
        if self.s.f:
            orc.lib().orc_free(C.byref(self.s))
