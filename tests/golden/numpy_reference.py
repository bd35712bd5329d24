"""Array-oriented numpy restatement of the reference's single-rank step.

A second, independently written restatement used only to cross-check the C
oracle (oracle/lbm_oracle.c): same reference semantics, different code
shape (whole-array operations instead of per-node loops). Every elementwise
operation is the same IEEE double operation in the same order as the
reference, so the two must agree bit for bit. Small grids only.

Reference: lbm.f90:24-227, initialization.f90:59-282, cart_mpi.f90:240-277
(and the _3d files).
"""
import numpy as np

G = 3


class NumpyLBM:
    def __init__(self, dim, nx, ny, nz, charlength, xpos, re, ome, dt, rho0):
        self.dim, self.nq = dim, (9 if dim == 2 else 27)
        self.nx, self.ny, self.nz = nx, ny, (nz if dim == 3 else 0)
        # DataInput (initialization.f90:65-81)
        self.charlength = charlength * nx
        self.pos = xpos * nx
        self.ome, self.rho0 = ome, rho0
        self.nu = (2.0 - ome) * dt / (6.0 * ome)
        self.uu = re * self.nu / self.charlength
        self.radius = self.charlength * 0.5
        self.L = [nx + 1, ny + 1] + ([nz + 1] if dim == 3 else [])
        self.P = [l + 2 * G for l in self.L]
        self.dy = self.P[0]
        self.dz = self.P[0] * self.P[1] if dim == 3 else 0
        self.N = int(np.prod(self.P))
        self._lattice()
        self._geometry()
        n, nq = self.N, self.nq
        self.f = np.zeros((n, nq))
        self.fb = np.zeros((n, nq))
        self.p = np.zeros(n)
        self.u = np.zeros((n, dim))

    # InitLattice (initialization.f90:112-123, _3d:108-122)
    def _lattice(self):
        nq, dim = self.nq, self.dim
        self.e = np.zeros((nq, dim), dtype=np.int64)
        self.t = np.zeros(nq)
        for iq in range(nq):
            if dim == 2:
                i, j = iq // 3 - 1, iq % 3 - 1
                self.e[iq] = (i, j)
                w = np.float32(4.0) * (np.float32(1.0) - np.float32(0.75) * np.float32(i * i))
                w = np.float32(w * (np.float32(1.0) - np.float32(0.75) * np.float32(j * j)))
                self.t[iq] = float(w) / 9.0
            else:
                k, i, j = iq // 9 - 1, (iq // 3) % 3 - 1, iq % 3 - 1
                self.e[iq] = (i, j, k)
                self.t[iq] = 8.0 / 4.0 ** (abs(i) + abs(j) + abs(k)) / 27.0
        self.off = self.e[:, 0] + self.dy * self.e[:, 1]
        if dim == 3:
            self.off = self.off + self.dz * self.e[:, 2]

    def _coords(self):
        idx = np.arange(self.N)
        X = idx % self.dy
        Y = (idx // self.dy) % self.P[1]
        Z = idx // self.dz if self.dim == 3 else np.zeros_like(idx)
        return X, Y, Z

    def _wrap_src(self):
        X, Y, Z = self._coords()
        w = lambda c, l: np.where(c < G, c + l, np.where(c >= l + G, c - l, c))
        src = w(X, self.L[0]) + self.dy * w(Y, self.L[1])
        if self.dim == 3:
            src = src + self.dz * w(Z, self.L[2])
        ghost = src != np.arange(self.N)
        return ghost, src

    # SetGeometry (initialization.f90:167-255, _3d:170-279)
    def _geometry(self):
        dim = self.dim
        X, Y, Z = self._coords()
        x, y, z = X - G, Y - G, Z - G
        interior = (x >= 0) & (x < self.L[0]) & (y >= 0) & (y < self.L[1])
        if dim == 3:
            interior &= (z >= 0) & (z < self.L[2])
        r2 = (x - self.pos) ** 2 + (y - self.ny / 2.0) ** 2
        if dim == 3:
            r2 = r2 + (z - self.nz / 2.0) ** 2
        geo = np.zeros(self.N, dtype=np.int64)
        geo[interior & (r2 > self.radius ** 2)] = 1
        self.ghost, self.wsrc = self._wrap_src()
        geo[self.ghost] = geo[self.wsrc[self.ghost]]
        self.geo = geo
        self.fluid_id = np.flatnonzero(interior & (geo == 1))
        # ring lists in loop order: positions x,y[,z] in [-1, n+2]
        # loop ranges of SetGeometry: positions -1 .. n+2 per dimension
        ring = (x >= -1) & (x <= self.L[0] + 1) & (y >= -1) & (y <= self.L[1] + 1)
        if dim == 3:
            ring &= (z >= -1) & (z <= self.L[2] + 1)
        ring &= ~interior
        self.bl = np.flatnonzero(ring & (x == -1))
        self.br = np.flatnonzero(ring & (x == self.nx + 1))
        if dim == 2:
            self.bd = np.flatnonzero(ring & (y == -1))
            self.bu = np.flatnonzero(ring & (y == self.ny + 1))
        else:
            self.bd = np.flatnonzero(ring & (z == -1))
            self.bu = np.flatnonzero(ring & (z == self.nz + 1))
        # obstacle cells: per x-row the first solid cell with a fluid probe
        scan = (x >= -1) & (x <= self.L[0] + 1) & (y >= -1) & (y <= self.L[1] + 1)
        if dim == 3:
            scan &= (z >= -1) & (z <= self.L[2] + 1)
        cand = np.flatnonzero(scan & (geo == 0))
        hit = np.zeros(cand.size, dtype=bool)
        for iq in range(self.nq):  # probes in iq order, stopping at the first hit
            pr = cand + self.e[iq, 0] + self.dy * (iq * dim + 1)
            if dim == 3:
                pr = pr + self.dz * (iq * dim + 2)
            live = ~hit
            assert np.all((pr[live] >= 0) & (pr[live] < self.N)), "probe leaves the geo array"
            hit[live] = geo[pr[live]] == 1
        cand = cand[hit]
        rows = cand // self.dy
        _, first = np.unique(rows, return_index=True)
        self.b_user = np.sort(cand[first])

    # InitUP (initialization.f90:259-282, _3d:282-308)
    def init_up(self, r_vec):
        ids = np.flatnonzero(self.interior_mask())
        r = 1.0 + (r_vec[ids % 100] - 0.5) * 2.0 * 0.2
        g = self.geo[ids].astype(np.float64)
        self.p[ids] = 0.0
        if self.dim == 2:
            y = (ids // self.dy - G).astype(np.float64)
            self.u[ids, 0] = self.uu * 4.0 * y * (self.ny - y) / float(self.ny * self.ny) * g * r
        else:
            z = (ids // self.dz - G).astype(np.float64)
            self.u[ids, 0] = self.uu * 4.0 * z * (self.nz - z) / float(self.nz * self.nz) * r * g
        self.u[ids, 1:] = 0.0

    def interior_mask(self):
        X, Y, Z = self._coords()
        m = (X >= G) & (X < self.L[0] + G) & (Y >= G) & (Y < self.L[1] + G)
        if self.dim == 3:
            m &= (Z >= G) & (Z < self.L[2] + G)
        return m

    def _feq(self, ids):
        u = self.u[ids]
        udu = np.zeros(ids.size)
        for k in range(self.dim):
            udu = udu + u[:, k] * u[:, k]
        out = np.empty((ids.size, self.nq))
        for iq in range(self.nq):
            edu = np.zeros(ids.size)
            for k in range(self.dim):
                edu = edu + float(self.e[iq, k]) * u[:, k]
            s = 3.0 * edu + 4.5 * (edu * edu) - 1.5 * udu
            out[:, iq] = self.t[iq] * (self.p[ids] * 3.0 + self.rho0 * s)
        return out

    def init_pdf(self):
        self.f[self.fluid_id] = self._feq(self.fluid_id)

    def collision(self):
        ids = self.fluid_id
        self.fb[ids] = (1.0 - self.ome) * self.f[ids] + self.ome * self._feq(ids)

    def boundary(self):
        fb = self.fb.reshape(-1)
        nq, n = self.nq, self.N
        F = self.fb
        F[self.ghost] = F[self.wsrc[self.ghost]]  # PassF, one rank

        def read(idx):
            v = np.full(idx.shape, np.nan)
            ok = (idx >= 0) & (idx < n * nq)
            v[ok] = fb[idx[ok]]
            return v

        rev = np.arange(nq)[::-1]
        # Up, Down, User loops; each cell is done before the next one
        for lst in (self.bu, self.bd, self.b_user):
            for c in lst:
                for iq in range(nq):
                    fb[c * nq + iq] = read(np.array([(c + 2 * self.off[iq]) * nq + rev[iq]]))[0]
        for c in self.bl:
            fb[c * nq:(c + 1) * nq] = fb[(c + 1) * nq:(c + 2) * nq]
        for c in self.br:
            for iq in range(nq):
                fb[c * nq + iq] = read(np.array([(c + self.off[iq]) * nq + iq]))[0]

    def propagation(self):
        ids = self.fluid_id
        for iq in range(self.nq):
            self.f[ids, iq] = self.fb[ids - self.off[iq], iq]

    def post_processing(self):
        ids = self.fluid_id
        f = self.f[ids]
        p = np.zeros(ids.size)
        u = np.zeros((ids.size, self.dim))
        for iq in range(self.nq):
            p = p + f[:, iq]
            for k in range(self.dim):
                u[:, k] = u[:, k] + f[:, iq] * float(self.e[iq, k])
        g = self.geo[ids].astype(np.float64)
        self.u[ids] = u / self.rho0 * g[:, None]
        self.p[ids] = p / 3.0 * g
        c = self.bl + 1
        if self.dim == 2:
            y = c // self.dy - G
            self.u[c, 0] = self.uu * self.rho0 * 4.0 * y * (self.ny - y).astype(np.float64) / float(self.ny * self.ny)
        else:
            z = c // self.dz - G
            self.u[c, 0] = self.uu * self.rho0 * 4.0 * z * (self.nz - z).astype(np.float64) / float(self.nz * self.nz)
        self.u[c, 1] = 0.0
        self.p[self.br - 1] = 0.0

    def monitor(self):
        ids = self.fluid_id[1:]
        v = np.sqrt(self.u[ids, 0] * self.u[ids, 0] + self.u[ids, 1] * self.u[ids, 1])
        return float(v.max()) if v.size else 0.0

    def run(self, iter0, nsteps, interv):
        log = []
        for it in range(iter0, iter0 + nsteps):
            if interv > 0 and it % interv == 0:
                log.append(self.monitor())
            self.collision()
            self.boundary()
            self.propagation()
            self.post_processing()
        return np.array(log)
