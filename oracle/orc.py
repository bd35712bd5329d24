"""ctypes front end of the CPU oracle (test infrastructure only).

Used by tests/, by the smoke check and by the benchmark's CPU-baseline leg as
the checker; the product path never imports it. Parity unpinned by the
reference (it has no tests or outputs to compare with); the oracle is pinned
by known-answer tests and an independent numpy restatement.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

_c_int, _c_dbl, _c_ll = C.c_int, C.c_double, C.c_longlong
_pd, _pi = C.POINTER(C.c_double), C.POINTER(C.c_int)


class OrcInput(C.Structure):
    _fields_ = [("dim", _c_int), ("nx", _c_int), ("ny", _c_int), ("nz", _c_int),
                ("charlength", _c_dbl), ("xpos", _c_dbl), ("re", _c_dbl),
                ("ome", _c_dbl), ("dt", _c_dbl), ("rho0", _c_dbl),
                ("max_t", _c_dbl), ("inter", _c_dbl)]


class OrcState(C.Structure):
    _fields_ = [("dim", _c_int), ("nq", _c_int), ("nx", _c_int), ("ny", _c_int), ("nz", _c_int),
                ("charlength", _c_dbl), ("pos", _c_dbl), ("re", _c_dbl), ("uu", _c_dbl),
                ("ma", _c_dbl), ("radius", _c_dbl),
                ("nu", _c_dbl), ("rho0", _c_dbl), ("dt", _c_dbl), ("ome", _c_dbl),
                ("tau", _c_dbl), ("t_intv", _c_dbl), ("inter", _c_dbl), ("max_t", _c_dbl),
                ("max_step", _c_int), ("interv", _c_int),
                ("L", _c_int * 3), ("dy", _c_int), ("dz", _c_int), ("array_size", _c_ll),
                ("t", _c_dbl * 27), ("e", _c_int * 81),
                ("f", _pd), ("fb", _pd), ("p", _pd), ("u", _pd),
                ("geo", _pi), ("fluid_id", _pi), ("bl", _pi), ("br", _pi), ("bu", _pi),
                ("bd", _pi), ("bf", _pi), ("bb", _pi), ("b_user", _pi),
                ("size_fluid", _c_int), ("l_size", _c_int), ("r_size", _c_int),
                ("u_size", _c_int), ("d_size", _c_int), ("f_size", _c_int),
                ("b_size", _c_int), ("user_size", _c_int),
                ("oob_reads", _c_ll), ("geom_error", _c_int), ("nthreads", _c_int),
                ("start", _c_int * 3)]


class OrcGroup(C.Structure):
    _fields_ = [("dim", _c_int), ("nprocs", _c_int), ("np", _c_int * 3), ("gl", _c_int * 3),
                ("cc", C.POINTER(_c_int * 3)), ("r", C.POINTER(OrcState))]


_lib = None
_lib_fma = None


def lib(contract=False):
    """The oracle library (contract: the build with a*b+c fused, see
    build.LIB_FMA)."""
    global _lib, _lib_fma
    if (_lib_fma if contract else _lib) is None:
        path = _build.build(contract=contract)
        L = C.CDLL(path)
        L.orc_read_input.argtypes = [C.c_char_p, _c_int, C.POINTER(OrcInput)]
        L.orc_setup.argtypes = [C.POINTER(OrcState), C.POINTER(OrcInput)]
        for name in ("orc_free", "orc_init_pdf", "orc_collision", "orc_boundary_condition",
                     "orc_propagation", "orc_post_processing"):
            getattr(L, name).argtypes = [C.POINTER(OrcState)]
        L.orc_init_up.argtypes = [C.POINTER(OrcState), _pd]
        L.orc_pass_f.argtypes = [C.POINTER(OrcState), _pd]
        L.orc_apply_bc.argtypes = [C.POINTER(OrcState), _pd]
        L.orc_monitor.argtypes = [C.POINTER(OrcState)]
        L.orc_monitor.restype = _c_dbl
        L.orc_run.argtypes = [C.POINTER(OrcState), _c_int, _c_int, _c_int, _pd]
        L.orc_r_vec.argtypes = [C.c_ulonglong, _pd]
        L.orc_forces.argtypes = [C.POINTER(OrcState), _pd]
        L.orc_forces.restype = _c_int
        L.orc_mass.argtypes = [C.POINTER(OrcState)]
        L.orc_mass.restype = _c_dbl
        L.orc_corrected_obstacles.argtypes = [C.POINTER(OrcState)]
        L.orc_bc_copies.argtypes = [C.POINTER(OrcState), _pd]
        L.orc_decompose.argtypes = [_c_int, C.POINTER(_c_int), _c_int, C.POINTER(_c_int)]
        L.orc_local_box.argtypes = [_c_int, C.POINTER(_c_int), C.POINTER(_c_int), C.POINTER(_c_int),
                                    C.POINTER(_c_int), C.POINTER(_c_int)]
        L.orc_group_setup.argtypes = [C.POINTER(OrcGroup), C.POINTER(OrcInput), _c_int]
        L.orc_setup_rank.argtypes = [C.POINTER(OrcState), C.POINTER(OrcInput), C.POINTER(_c_int),
                                     C.POINTER(_c_int)]
        L.orc_obstacle_scan.argtypes = [C.POINTER(OrcState)]
        for name in ("orc_group_free", "orc_group_pass_f", "orc_group_init_pdf"):
            getattr(L, name).argtypes = [C.POINTER(OrcGroup)]
        L.orc_group_init_up.argtypes = [C.POINTER(OrcGroup), _pd]
        L.orc_group_monitor.argtypes = [C.POINTER(OrcGroup)]
        L.orc_group_monitor.restype = _c_dbl
        L.orc_group_run.argtypes = [C.POINTER(OrcGroup), _c_int, _c_int, _c_int, _pd]
        if contract:
            _lib_fma = L
        else:
            _lib = L
    return _lib_fma if contract else _lib


def make_input(dim, nx, ny, nz=0, charlength=0.125, xpos=0.25, re=100.0, ome=1.8,
               dt=1.0, rho0=1.0, max_t=0.0, inter=0.0):
    """The four input.in lines as a structure (values as they appear in the file)."""
    return OrcInput(dim, nx, ny, nz, charlength, xpos, re, ome, dt, rho0, max_t, inter)


def read_input(path, dim):
    inp = OrcInput()
    rc = lib().orc_read_input(os.fsencode(path), dim, C.byref(inp))
    if rc != 0:
        raise ValueError("oracle could not parse %s (rc=%d)" % (path, rc))
    return inp


def r_vec(seed=12345):
    out = np.zeros(100, dtype=np.float64)
    lib().orc_r_vec(seed, out.ctypes.data_as(_pd))
    return out


class Oracle:
    """One reference-layout state advanced by the serial reference program."""

    def __init__(self, inp, nthreads=1, allow_geom_error=False, _state=None, _owner=None,
                 contract=False):
        self._owner = _owner  # a rank of an OracleGroup: the group owns the state
        # contract: the build with a*b+c fused into multiply-adds (build.LIB_FMA)
        self._L = lib(contract)
        if _state is not None:
            self.s = _state
        else:
            self.s = OrcState()
            rc = self._L.orc_setup(C.byref(self.s), C.byref(inp))
            if rc != 0 and not (rc == -2 and allow_geom_error):
                self._L.orc_free(C.byref(self.s))
                raise ValueError("oracle setup failed (rc=%d)" % rc)
        self.s.nthreads = nthreads
        s = self.s
        n, nq, dim = s.array_size, s.nq, s.dim
        self.f = np.ctypeslib.as_array(s.f, shape=(n * nq,))
        self.fb = np.ctypeslib.as_array(s.fb, shape=(n * nq,))
        self.p = np.ctypeslib.as_array(s.p, shape=(n,))
        self.u = np.ctypeslib.as_array(s.u, shape=(n * dim,))
        self.geo = np.ctypeslib.as_array(s.geo, shape=(n,))

    def _list(self, name, size):
        size = int(size)
        if size == 0:
            return np.zeros(0, dtype=np.int32)
        return np.ctypeslib.as_array(getattr(self.s, name), shape=(size,)).copy()

    @property
    def lists(self):
        s = self.s
        return dict(fluid_id=self._list("fluid_id", s.size_fluid), bl=self._list("bl", s.l_size),
                    br=self._list("br", s.r_size), bu=self._list("bu", s.u_size),
                    bd=self._list("bd", s.d_size), bf=self._list("bf", s.f_size),
                    bb=self._list("bb", s.b_size), b_user=self._list("b_user", s.user_size))

    def use_corrected_obstacles(self):
        """Replace b_user with the corrected-physics list (every interior
        solid node with a fluid neighbour); not the reference's rule."""
        self._L.orc_corrected_obstacles(C.byref(self.s))

    @property
    def t(self):
        return np.array(self.s.t[:self.s.nq])

    @property
    def e(self):
        return np.array(self.s.e[:self.s.nq * self.s.dim], dtype=np.int32)

    def init_up(self, rv):
        rv = np.ascontiguousarray(rv, dtype=np.float64)
        self._L.orc_init_up(C.byref(self.s), rv.ctypes.data_as(_pd))

    def init_pdf(self):
        self._L.orc_init_pdf(C.byref(self.s))

    def collision(self):
        self._L.orc_collision(C.byref(self.s))

    def boundary_condition(self):
        self._L.orc_boundary_condition(C.byref(self.s))

    def propagation(self):
        self._L.orc_propagation(C.byref(self.s))

    def post_processing(self):
        self._L.orc_post_processing(C.byref(self.s))

    def monitor(self):
        return self._L.orc_monitor(C.byref(self.s))

    def forces(self):
        """Momentum-exchange force on the obstacle after the last BC."""
        F = np.zeros(3)
        n = self._L.orc_forces(C.byref(self.s), F.ctypes.data_as(_pd))
        return F[:self.s.dim], n

    def mass(self):
        return self._L.orc_mass(C.byref(self.s))

    def apply_bc(self, a):
        assert a.dtype == np.float64 and a.flags.c_contiguous and a.size == self.fb.size
        self._L.orc_apply_bc(C.byref(self.s), a.ctypes.data_as(_pd))

    def run(self, iter0, nsteps, interv):
        nmon = 0
        if interv > 0:
            nmon = sum(1 for it in range(iter0, iter0 + nsteps) if it % interv == 0)
        log = np.zeros(max(nmon, 1), dtype=np.float64)
        m = self._L.orc_run(C.byref(self.s), iter0, nsteps, interv, log.ctypes.data_as(_pd))
        assert m == nmon
        return log[:nmon]

    def bc_copies(self, a=None):
        """BoundaryCondition after PassF (the rank's own copies) on fb or a."""
        a = self.fb if a is None else a
        self._L.orc_bc_copies(C.byref(self.s), a.ctypes.data_as(_pd))

    @property
    def start(self):
        return tuple(self.s.start[:self.s.dim])

    @property
    def local_length(self):
        return tuple(self.s.L[:self.s.dim])

    def close(self):
        if self._owner is None and self.s.f:
            self._L.orc_free(C.byref(self.s))

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def decompose(dim, gl, nprocs):
    """SetCartesian: ranks per dimension for global lengths gl (n+1 each)."""
    g = (_c_int * 3)(*(list(gl) + [1] * (3 - len(gl))))
    np_ = (_c_int * 3)()
    lib().orc_decompose(dim, g, nprocs, np_)
    return tuple(np_[:dim])


def local_box(dim, gl, nps, cc):
    """SetLocalLength: (local_length, local_start) of the rank at cc."""
    pad = lambda v: (_c_int * 3)(*(list(v) + [1] * (3 - len(v))))
    L = (_c_int * 3)()
    st = (_c_int * 3)()
    rc = lib().orc_local_box(dim, pad(gl), pad(nps), pad(list(cc) + [0] * (3 - len(cc))), L, st)
    if rc != 0:
        raise ValueError("local length below the ghost width")
    return tuple(L[:dim]), tuple(st[:dim])


class OracleGroup:
    """The reference run on nprocs MPI ranks, all ranks in one process."""

    def __init__(self, inp, nprocs, nthreads=1, allow_geom_error=False):
        self.g = OrcGroup()
        rc = lib().orc_group_setup(C.byref(self.g), C.byref(inp), nprocs)
        if rc != 0 and not (rc == -2 and allow_geom_error):
            lib().orc_group_free(C.byref(self.g))
            raise ValueError("oracle group setup failed (rc=%d)" % rc)
        self.nprocs = nprocs
        self.ranks = [Oracle(None, nthreads, _state=self.g.r[a], _owner=self) for a in range(nprocs)]

    @property
    def np(self):
        return tuple(self.g.np[:self.g.dim])

    def coords(self, a):
        return tuple(self.g.cc[a][:self.g.dim])

    def init_up(self, r_vecs):
        rv = np.ascontiguousarray(np.asarray(r_vecs, dtype=np.float64).reshape(self.nprocs, 100))
        lib().orc_group_init_up(C.byref(self.g), rv.ctypes.data_as(_pd))

    def init_pdf(self):
        lib().orc_group_init_pdf(C.byref(self.g))

    def pass_f(self):
        lib().orc_group_pass_f(C.byref(self.g))

    def monitor(self):
        return lib().orc_group_monitor(C.byref(self.g))

    def run(self, iter0, nsteps, interv):
        nmon = sum(1 for it in range(iter0, iter0 + nsteps) if interv > 0 and it % interv == 0)
        log = np.zeros(max(nmon, 1), dtype=np.float64)
        m = lib().orc_group_run(C.byref(self.g), iter0, nsteps, interv, log.ctypes.data_as(_pd))
        assert m == nmon
        return log[:nmon]

    def close(self):
        if self.g.r:
            self.ranks = []
            lib().orc_group_free(C.byref(self.g))

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
