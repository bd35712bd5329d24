"""Python front end of libimexlb (ctypes over the C ABI in include/imexlb.h).

The library is the product: a C ABI whose calls replace the per-timestep
subroutines IMEXLB-1.0's main program calls (main.f90:48-63). This module only
loads it and converts numpy arrays; it has no compute path of its own and
raises if the compiled library is missing.

    cfg = read_input("input_3d.in", dim=3)        # DataInput + one-rank MPISetup
    setup = Setup(cfg)                            # InitLattice, SetGeometry, InitUP
    with Solver(cfg) as s:
        s.set_geometry(setup)
        s.upload(setup.f, setup.fb, setup.p, setup.u)
        s.init_pdf()                              # InitPDF on the device
        umax = s.step(0, 1000, cfg.interv)        # Monitor + Collision..PostProcessing
        f, fb, p, u = s.download()
"""
import ctypes as C
import os

import numpy as np

_PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(_PKG, "_build", "libimexlb.so")

IMEXLB_OK = 0
ERR_ARG, ERR_CUDA, ERR_STATE, ERR_GEOMETRY, ERR_UNSUPPORTED, ERR_NOMEM = -1, -2, -3, -4, -5, -6
ERR_DIVERGED, ERR_TIMEOUT = -7, -8
BATCH_LOCKSTEP, BATCH_PERSISTENT = 0, 1
FP64, FP64_FAST, FP32, BF16, FP16, FIX64 = 0, 1, 2, 3, 4, 5

_c_int, _c_dbl, _c_ll = C.c_int, C.c_double, C.c_longlong
_pd, _pi = C.POINTER(C.c_double), C.POINTER(C.c_int)


class ImexlbError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("imexlb error %d: %s" % (code, msg))
        self.code = code


class Desc(C.Structure):
    _fields_ = [("dim", _c_int), ("nq", _c_int), ("ghost", _c_int),
                ("nx", _c_int), ("ny", _c_int), ("nz", _c_int),
                ("local_length", _c_int * 3), ("local_start", _c_int * 3),
                ("dy", _c_int), ("dz", _c_int),
                ("ome", _c_dbl), ("rho0", _c_dbl), ("uu", _c_dbl),
                ("t", _c_dbl * 27), ("e", _c_int * 81),
                ("precision", _c_int), ("device", _c_int)]


class Info(C.Structure):
    _fields_ = [("array_size", _c_ll), ("interior", _c_ll), ("size_fluid", _c_ll),
                ("n_fill", _c_ll), ("n_user", _c_ll), ("n_links", _c_ll),
                ("device_bytes", _c_ll)]


KERNEL_STEP, KERNEL_FILL, KERNEL_FIRST, KERNEL_OTHER = 0, 1, 2, 3
FILL_KERNEL, FILL_FUSED = 0, 1


class Profile(C.Structure):
    _fields_ = [("launches", _c_ll * 4), ("ms", _c_dbl * 4)]


class ConvDesc(C.Structure):
    _fields_ = [("n", _c_int), ("hin", _c_int), ("win", _c_int), ("cin", _c_int),
                ("hout", _c_int), ("wout", _c_int), ("cout", _c_int), ("cout_store", _c_int),
                ("stride", _c_int), ("upsample", _c_int)]


class Config(C.Structure):
    _fields_ = [("dim", _c_int), ("nx", _c_int), ("ny", _c_int), ("nz", _c_int),
                ("charlength_in", _c_dbl), ("xpos_in", _c_dbl), ("re", _c_dbl),
                ("ome", _c_dbl), ("dt", _c_dbl), ("rho0", _c_dbl),
                ("max_t", _c_dbl), ("inter", _c_dbl),
                ("charlength", _c_dbl), ("pos", _c_dbl), ("nu", _c_dbl), ("t_intv", _c_dbl),
                ("uu", _c_dbl), ("tau", _c_dbl), ("ma", _c_dbl), ("radius", _c_dbl),
                ("interv", _c_int), ("max_step", _c_int),
                ("local_length", _c_int * 3), ("local_start", _c_int * 3),
                ("dy", _c_int), ("dz", _c_int), ("array_size", _c_ll),
                ("yoff", _c_dbl)]

    @property
    def nq(self):
        return 9 if self.dim == 2 else 27

    @property
    def nodes(self):
        n = (self.nx + 1) * (self.ny + 1)
        return n * (self.nz + 1) if self.dim == 3 else n


_lib = None

# name: (restype, argtypes) for every symbol of include/imexlb.h,
# include/imexlb_host.h, include/imexlb_testing.h and include/imexlb_nn.h.
_SIGS = {
    "imexlb_create": (_c_int, [C.POINTER(C.c_void_p), C.POINTER(Desc)]),
    "imexlb_set_geometry": (_c_int, [C.c_void_p, _pi, _pi, _c_int, _pi, _c_int, _pi, _c_int,
                                     _pi, _c_int, _pi, _c_int, _pi, _c_int]),
    "imexlb_upload": (_c_int, [C.c_void_p, _pd, _pd, _pd, _pd]),
    "imexlb_init_pdf": (_c_int, [C.c_void_p]),
    "imexlb_step": (_c_int, [C.c_void_p, _c_int, _c_int, _c_int, _pd]),
    "imexlb_download": (_c_int, [C.c_void_p, _pd, _pd, _pd, _pd]),
    "imexlb_observe": (_c_int, [C.c_void_p, _pd, _pd]),
    "imexlb_step_observed": (_c_int, [C.c_void_p, _c_int, _c_int, _c_int, _pd, _c_int, _pd]),
    "imexlb_get_info": (_c_int, [C.c_void_p, C.POINTER(Info)]),
    "imexlb_get_stream": (_c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    "imexlb_fp64_splits": (_c_int, []),
    "imexlb_set_fp64_split": (_c_int, [C.c_void_p, _c_int]),
    "imexlb_fp64_fma_rate": (_c_int, [_c_int, _pd]),
    "imexlb_set_fill_mode": (_c_int, [C.c_void_p, _c_int]),
    "imexlb_set_watchdog": (_c_int, [C.c_void_p, _c_int]),
    "imexlb_get_fill_mode": (_c_int, [C.c_void_p, _pi]),
    "imexlb_profile_reset": (_c_int, [C.c_void_p, _c_int]),
    "imexlb_profile_read": (_c_int, [C.c_void_p, C.POINTER(Profile)]),
    "imexlb_destroy": (None, [C.c_void_p]),
    "imexlb_batch_create": (_c_int, [C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), _c_int]),
    "imexlb_batch_tune": (_c_int, [C.c_void_p, _c_int, C.POINTER(_c_int)]),
    "imexlb_batch_step": (_c_int, [C.c_void_p, _c_int, _pi]),
    "imexlb_batch_destroy": (None, [C.c_void_p]),
    "imexlb_batch_set_mode": (_c_int, [C.c_void_p, _c_int]),
    "imexlb_testing_batch_stall": (_c_int, [C.c_void_p, _c_int, _c_dbl]),
    "imexlb_testing_set_staged_kernel": (_c_int, [C.c_void_p, _c_int]),
    "imexlb_testing_stage_stall": (_c_int, [C.c_void_p, _c_dbl]),
    "imexlb_batch_last_error": (C.c_char_p, [C.c_void_p]),
    "imexlb_sample": (_c_int, [C.c_void_p, _c_int, _c_int, C.POINTER(C.c_float)]),
    "imexlb_init_state": (_c_int, [C.c_void_p, _pd]),
    "imexlb_group_create": (_c_int, [C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), _c_int]),
    "imexlb_group_step": (_c_int, [C.c_void_p, _c_int, _c_int, _c_int, _pd]),
    "imexlb_group_destroy": (None, [C.c_void_p]),
    "imexlb_group_last_error": (C.c_char_p, [C.c_void_p]),
    "imexlb_nn_conv_fwd": (_c_int, [C.POINTER(ConvDesc), C.c_void_p, C.c_void_p, C.c_void_p, _c_int,
                                    C.c_void_p, C.c_void_p, C.c_void_p]),
    "imexlb_nn_act_grad": (_c_int, [C.c_void_p, C.c_void_p, _c_ll, _c_int, _c_int, C.c_void_p,
                                    C.c_void_p, C.c_void_p]),
    "imexlb_nn_conv_bwd_data": (_c_int, [C.POINTER(ConvDesc), C.c_void_p, C.c_void_p, C.c_void_p,
                                         C.c_void_p, C.c_void_p, C.c_void_p]),
    "imexlb_nn_conv_bwd_weight": (_c_int, [C.POINTER(ConvDesc), C.c_void_p, C.c_void_p, C.c_void_p,
                                           C.c_void_p]),
    "imexlb_nn_mse": (_c_int, [C.c_void_p, C.c_void_p, C.c_void_p, _c_ll, _c_int, _c_int, C.c_void_p,
                               C.c_void_p, C.c_void_p]),
    "imexlb_nn_adam": (_c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, _c_ll,
                                C.c_float, C.c_float, C.c_float, C.c_float, _c_int, C.c_float,
                                C.c_void_p]),
    "imexlb_nn_status": (_c_int, [C.POINTER(_c_int)]),
    "imexlb_monitor_noalloc": (_c_int, [_c_int, C.c_void_p, C.c_void_p, _c_int, C.c_void_p,
                                        C.c_void_p]),
    "imexlb_last_error": (C.c_char_p, [C.c_void_p]),
    "imexlb_version": (C.c_char_p, []),
    "imexlb_host_read_input": (_c_int, [C.c_char_p, _c_int, C.POINTER(Config)]),
    "imexlb_host_derive": (_c_int, [C.POINTER(Config)]),
    "imexlb_host_lattice": (_c_int, [_c_int, _pd, _pi]),
    "imexlb_host_list_capacity": (_c_int, [C.POINTER(Config), C.POINTER(_c_ll)]),
    "imexlb_host_set_geometry": (_c_int, [C.POINTER(Config), _pi, _pi, _pi, _pi, _pi, _pi, _pi,
                                          _pi, _pi, _pi]),
    "imexlb_host_r_vec": (None, [C.c_ulonglong, _pd]),
    "imexlb_host_obstacle_cells": (_c_int, [C.POINTER(Config), _pi, _pi, _pi]),
    "imexlb_device_set_geometry": (_c_int, [C.POINTER(Config), _c_int, _pi, _pi, _pi, _pi, _pi, _pi,
                                            _pi, _pi, _pi, _pi]),
    "imexlb_host_geometry_lists": (_c_int, [C.POINTER(Config), _pi, _pi, _pi, _pi, _pi, _pi, _pi, _pi,
                                            _pi]),
    "imexlb_host_group_pass_int": (_c_int, [C.POINTER(Config), _pi, _c_int, C.POINTER(_pi)]),
    "imexlb_host_obstacle_scan": (_c_int, [C.POINTER(Config), _pi, _pi, _pi]),
    "imexlb_host_decompose": (_c_int, [_c_int, _pi, _c_int, _pi]),
    "imexlb_host_rank_layout": (_c_int, [C.POINTER(Config), _pi, _c_int]),
    "imexlb_host_init_up": (_c_int, [C.POINTER(Config), _pi, _pd, _pd, _pd]),
    "imexlb_host_write_plt": (_c_int, [C.POINTER(Config), C.c_char_p, _c_int, _c_int, _pd, _pd, _pi,
                                       _c_int]),
    "imexlb_host_make_desc": (_c_int, [C.POINTER(Config), _c_int, _c_int, C.POINTER(Desc)]),
    "imexlb_testing_resolve_bc": (_c_ll, [C.POINTER(Desc), _pi, _c_int, _pi, _c_int, _pi, _c_int,
                                          _pi, _c_int, _pi, _c_int, _pi, _c_int, _pd, _pd]),
    "imexlb_testing_fused_pull": (_c_ll, [C.POINTER(Desc), _pi, _c_int, _pi, _c_int, _pi, _c_int,
                                          _pi, _c_int, _pi, _c_int, _pi, _c_int, _pd, _pd, _pd,
                                          _pd, C.POINTER(_c_ll)]),
}


def lib():
    """Load libimexlb.so (built in-tree by __graft_entry__.build()); raise if absent."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libimexlb.so is not built (%s); run __graft_entry__.build()" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def symbols():
    return list(_SIGS)


def _p(a, ct):
    return a.ctypes.data_as(C.POINTER(ct)) if a is not None else None


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


# ----------------------------------------------------------------------------
# Host setup (include/imexlb_host.h)
# ----------------------------------------------------------------------------

def fp64_splits():
    """Number of FP64 step-kernel variants (see Solver.set_fp64_split)."""
    return lib().imexlb_fp64_splits()


def read_input(path, dim):
    """DataInput: parse input.in / input_3d.in and derive the rest."""
    c = Config()
    rc = lib().imexlb_host_read_input(os.fsencode(path), dim, C.byref(c))
    if rc != IMEXLB_OK:
        raise ImexlbError(rc, "cannot read input file %s" % path)
    return c


def make_config(dim, nx, ny, nz=0, charlength=0.125, xpos=0.25, re=100.0, ome=1.8, dt=1.0,
                rho0=1.0, max_t=0.0, inter=0.0, yoff=0.0):
    """Config from the values of the four input.in lines (yoff: obstacle
    centre offset in y, an extension; 0 is the reference geometry)."""
    c = Config()
    c.yoff = yoff
    c.dim, c.nx, c.ny, c.nz = dim, nx, ny, nz
    c.charlength_in, c.xpos_in, c.re = charlength, xpos, re
    c.ome, c.dt, c.rho0 = ome, dt, rho0
    c.max_t, c.inter = max_t, inter
    rc = lib().imexlb_host_derive(C.byref(c))
    if rc != IMEXLB_OK:
        raise ImexlbError(rc, "invalid configuration")
    return c


def lattice(dim):
    nq = 9 if dim == 2 else 27
    t = np.zeros(nq)
    e = np.zeros(nq * dim, dtype=np.int32)
    lib().imexlb_host_lattice(dim, _p(t, C.c_double), _p(e, C.c_int))
    return t, e


def r_vec(seed=12345):
    out = np.zeros(100)
    lib().imexlb_host_r_vec(seed, _p(out, C.c_double))
    return out


class Setup:
    """SetGeometry + InitUP on the host, arrays in the reference layout.

    f and fb start at zero (fresh allocation, as the reference's arrays are in
    practice); call Solver.init_pdf() for InitPDF on the device.

    physics="corrected" replaces the reference's obstacle list (at most one
    cell per x-row, found by its odd neighbour probe) with every solid cell
    that has a fluid neighbour (imexlb_host_obstacle_cells): a mode apart
    from the reference, whose results it does not reproduce.
    """

    LISTS = ("fluid_id", "bl", "br", "bu", "bd", "bf", "bb", "b_user")

    def __init__(self, cfg, seed=12345, rv=None, physics="reference", device=None,
                 state=True):
        """device: an ordinal to run SetGeometry on that CUDA device
        (imexlb_device_set_geometry, same results) instead of the host.
        state=False leaves out the f, fb, p, u arrays and InitUP (for callers
        that compute the initial state on the device)."""
        if physics not in ("reference", "corrected"):
            raise ValueError("physics is 'reference' or 'corrected'")
        L = lib()
        self.cfg = cfg
        n = cfg.array_size
        caps = (C.c_longlong * 8)()
        L.imexlb_host_list_capacity(C.byref(cfg), caps)
        self.geo = np.zeros(n, dtype=np.int32)
        bufs = [np.zeros(max(int(c), 1), dtype=np.int32) for c in caps]
        sizes = (C.c_int * 8)()
        if device is None:
            rc = L.imexlb_host_set_geometry(C.byref(cfg), _p(self.geo, C.c_int),
                                            *[_p(b, C.c_int) for b in bufs], sizes)
        else:
            rc = L.imexlb_device_set_geometry(C.byref(cfg), int(device), _p(self.geo, C.c_int),
                                              *[_p(b, C.c_int) for b in bufs], sizes)
            if rc == ERR_CUDA:
                raise ImexlbError(rc, L.imexlb_last_error(None).decode())
        # the reference rule's probe may leave geo on small 3D grids; the
        # corrected rule does not probe there
        if rc != IMEXLB_OK and not (physics == "corrected" and rc == ERR_GEOMETRY):
            raise ImexlbError(rc, "SetGeometry failed")
        for name, b, s in zip(self.LISTS, bufs, sizes):
            setattr(self, name, b[:s].copy())
        self.physics = physics
        if physics == "corrected":
            user = np.zeros(n, dtype=np.int32)
            nu = C.c_int()
            rc = L.imexlb_host_obstacle_cells(C.byref(cfg), _p(self.geo, C.c_int), _p(user, C.c_int),
                                              C.byref(nu))
            if rc != IMEXLB_OK:
                raise ImexlbError(rc, "obstacle cells failed")
            self.b_user = user[:nu.value].copy()
        nq, dim = cfg.nq, cfg.dim
        self.r_vec = r_vec(seed) if rv is None else _f64(rv)
        if not state:
            return
        self.f = np.zeros(n * nq)
        self.fb = np.zeros(n * nq)
        self.p = np.zeros(n)
        self.u = np.zeros(n * dim)
        rc = L.imexlb_host_init_up(C.byref(cfg), _p(self.geo, C.c_int), _p(self.r_vec, C.c_double),
                                   _p(self.p, C.c_double), _p(self.u, C.c_double))
        if rc != IMEXLB_OK:
            raise ImexlbError(rc, "InitUP failed")


def decompose(dim, gl, nprocs):
    """SetCartesian: ranks per dimension for nprocs ranks, gl = n+1 each."""
    g = (C.c_int * 3)(*(list(gl) + [1] * (3 - len(gl))))
    out = (C.c_int * 3)()
    rc = lib().imexlb_host_decompose(dim, g, nprocs, out)
    if rc != IMEXLB_OK:
        raise ImexlbError(rc, "decompose failed")
    return tuple(out[:dim])


def rank_config(cfg, nps, rank):
    """A copy of a derived config with MPI rank `rank`'s local box."""
    c = Config.from_buffer_copy(cfg)
    n = (C.c_int * 3)(*(list(nps) + [1] * (3 - len(nps))))
    rc = lib().imexlb_host_rank_layout(C.byref(c), n, rank)
    if rc != IMEXLB_OK:
        raise ImexlbError(rc, "rank %d: local length below the ghost width" % rank)
    return c


class RankSetup:
    """One rank's SetGeometry / InitUP arrays (reference layout, local box)."""


class GroupSetup:
    """SetGeometry and InitUP of the reference run on nprocs MPI ranks: per
    rank the geometry lists of its box, PassInt(geo) across the ranks, the
    rank's own obstacle scan, and InitUP with the rank's own draws (r_vecs[r];
    default: seeds seed + r)."""

    LISTS = Setup.LISTS

    def __init__(self, cfg, nprocs, seed=12345, r_vecs=None, allow_geom_error=False):
        L = lib()
        self.cfg = cfg
        gl = [cfg.nx + 1, cfg.ny + 1] + ([cfg.nz + 1] if cfg.dim == 3 else [])
        self.np = decompose(cfg.dim, gl, nprocs)
        self.ranks = []
        for r in range(nprocs):
            rs = RankSetup()
            rs.cfg = rank_config(cfg, self.np, r)
            n = rs.cfg.array_size
            caps = (C.c_longlong * 8)()
            L.imexlb_host_list_capacity(C.byref(rs.cfg), caps)
            rs.geo = np.zeros(n, dtype=np.int32)
            bufs = [np.zeros(max(int(c), 1), dtype=np.int32) for c in caps[:7]]
            sizes = (C.c_int * 7)()
            rc = L.imexlb_host_geometry_lists(C.byref(rs.cfg), _p(rs.geo, C.c_int),
                                              *[_p(b, C.c_int) for b in bufs], sizes)
            if rc != IMEXLB_OK:
                raise ImexlbError(rc, "rank %d: geometry failed" % r)
            for name, b, k in zip(self.LISTS[:7], bufs, sizes):
                setattr(rs, name, b[:k].copy())
            self.ranks.append(rs)
        geos = (_pi * nprocs)(*[_p(rs.geo, C.c_int) for rs in self.ranks])
        n3 = (C.c_int * 3)(*(list(self.np) + [1] * (3 - len(self.np))))
        rc = L.imexlb_host_group_pass_int(C.byref(cfg), n3, nprocs, geos)
        if rc != IMEXLB_OK:
            raise ImexlbError(rc, "PassInt across ranks failed")
        self.geom_error = False
        for r, rs in enumerate(self.ranks):
            user = np.zeros(rs.cfg.array_size, dtype=np.int32)
            nu = C.c_int()
            rc = L.imexlb_host_obstacle_scan(C.byref(rs.cfg), _p(rs.geo, C.c_int), _p(user, C.c_int),
                                             C.byref(nu))
            if rc == ERR_GEOMETRY:
                self.geom_error = True
                if not allow_geom_error:
                    raise ImexlbError(rc, "rank %d: the obstacle probe leaves the geo array" % r)
            elif rc != IMEXLB_OK:
                raise ImexlbError(rc, "obstacle scan failed")
            rs.b_user = user[:nu.value].copy()
            rs.r_vec = r_vec(seed + r) if r_vecs is None else _f64(r_vecs[r])
            n, nq, dim = rs.cfg.array_size, cfg.nq, cfg.dim
            rs.f = np.zeros(n * nq)
            rs.fb = np.zeros(n * nq)
            rs.p = np.zeros(n)
            rs.u = np.zeros(n * dim)
            rc = L.imexlb_host_init_up(C.byref(rs.cfg), _p(rs.geo, C.c_int), _p(rs.r_vec, C.c_double),
                                       _p(rs.p, C.c_double), _p(rs.u, C.c_double))
            if rc != IMEXLB_OK:
                raise ImexlbError(rc, "InitUP failed")


def write_plt(cfg, path, count, iteration, p, u, fluid_id):
    """WriteBinary: the reference's Tecplot binary file of the state."""
    p, u, fid = _f64(p), _f64(u), _i32(fluid_id)
    rc = lib().imexlb_host_write_plt(C.byref(cfg), os.fsencode(path), count, iteration,
                                     _p(p, C.c_double), _p(u, C.c_double), _p(fid, C.c_int), len(fid))
    if rc != IMEXLB_OK:
        raise ImexlbError(rc, "cannot write %s" % path)


def make_desc(cfg, precision=FP64, device=0):
    d = Desc()
    rc = lib().imexlb_host_make_desc(C.byref(cfg), precision, device, C.byref(d))
    if rc != IMEXLB_OK:
        raise ImexlbError(rc, "make_desc failed")
    return d


def resolve_bc(desc, lists, a):
    """Host-only: the library's boundary map applied to an fb-shaped array."""
    a = _f64(a)
    out = np.empty_like(a)
    g = {k: _i32(v) for k, v in lists.items()}
    n = lib().imexlb_testing_resolve_bc(
        C.byref(desc), _p(g["fluid_id"], C.c_int), len(g["fluid_id"]), _p(g["bl"], C.c_int),
        len(g["bl"]), _p(g["br"], C.c_int), len(g["br"]), _p(g["bu"], C.c_int), len(g["bu"]),
        _p(g["bd"], C.c_int), len(g["bd"]), _p(g["b_user"], C.c_int), len(g["b_user"]),
        _p(a, C.c_double), _p(out, C.c_double))
    return out, int(n)


def fp64_fma_rate(device=0):
    """FP64 fused multiply-adds per second of the device (short kernel)."""
    v = _c_dbl(0.0)
    rc = lib().imexlb_fp64_fma_rate(int(device), C.byref(v))
    if rc != IMEXLB_OK:
        raise ImexlbError(rc, "imexlb_fp64_fma_rate")
    return v.value


def fused_pull(desc, lists, cur, prev):
    """Host-only: one step's pulls (device SoA layout) with the boundary
    copies as a separate program and as the fused plan. Returns (pulled
    separate, pulled fused or None, records)."""
    cur, prev = _f64(cur), _f64(prev)
    a, b = np.empty_like(cur), np.empty_like(cur)
    nrec = _c_ll(0)
    g = {k: _i32(v) for k, v in lists.items()}
    rc = lib().imexlb_testing_fused_pull(
        C.byref(desc), _p(g["fluid_id"], C.c_int), len(g["fluid_id"]), _p(g["bl"], C.c_int),
        len(g["bl"]), _p(g["br"], C.c_int), len(g["br"]), _p(g["bu"], C.c_int), len(g["bu"]),
        _p(g["bd"], C.c_int), len(g["bd"]), _p(g["b_user"], C.c_int), len(g["b_user"]),
        _p(cur, C.c_double), _p(prev, C.c_double), _p(a, C.c_double), _p(b, C.c_double),
        C.byref(nrec))
    if rc < 0:
        raise ImexlbError(int(rc), "imexlb_testing_fused_pull")
    return a, (b if rc == 1 else None), int(nrec.value)


# ----------------------------------------------------------------------------
# Device solver (include/imexlb.h)
# ----------------------------------------------------------------------------

class Solver:
    """One libimexlb handle: the per-timestep lbm-module calls on one GPU."""

    def __init__(self, cfg_or_desc, precision=FP64, device=0):
        L = lib()
        desc = cfg_or_desc if isinstance(cfg_or_desc, Desc) else make_desc(cfg_or_desc, precision, device)
        self.desc = desc
        self.dim, self.nq = desc.dim, desc.nq
        h = C.c_void_p()
        rc = L.imexlb_create(C.byref(h), C.byref(desc))
        if rc != IMEXLB_OK:
            raise ImexlbError(rc, L.imexlb_last_error(None).decode())
        self.h = h
        self.n = None

    def _check(self, rc):
        if rc != IMEXLB_OK:
            raise ImexlbError(rc, lib().imexlb_last_error(self.h).decode())

    def set_geometry(self, setup=None, geo=None, **lists):
        if setup is not None:
            geo = setup.geo
            lists = {k: getattr(setup, k) for k in Setup.LISTS}
        g = _i32(geo)
        ls = {k: _i32(lists.get(k, np.zeros(0, dtype=np.int32))) for k in
              ("fluid_id", "bl", "br", "bu", "bd", "b_user")}
        self._keep = (g, ls)
        self.n = g.size
        self._check(lib().imexlb_set_geometry(
            self.h, _p(g, C.c_int), _p(ls["fluid_id"], C.c_int), len(ls["fluid_id"]),
            _p(ls["bl"], C.c_int), len(ls["bl"]), _p(ls["br"], C.c_int), len(ls["br"]),
            _p(ls["bu"], C.c_int), len(ls["bu"]), _p(ls["bd"], C.c_int), len(ls["bd"]),
            _p(ls["b_user"], C.c_int), len(ls["b_user"])))

    def upload(self, f, fb, p, u):
        f, fb, p, u = _f64(f), _f64(fb), _f64(p), _f64(u)
        self._check(lib().imexlb_upload(self.h, _p(f, C.c_double), _p(fb, C.c_double),
                                        _p(p, C.c_double), _p(u, C.c_double)))

    def upload_ptr(self, f, fb, p, u):
        """Upload from raw host addresses (e.g. pinned buffers)."""
        self._check(lib().imexlb_upload(self.h, C.cast(f, _pd), C.cast(fb, _pd), C.cast(p, _pd),
                                        C.cast(u, _pd)))

    def init_pdf(self):
        self._check(lib().imexlb_init_pdf(self.h))

    def step(self, iter0, nsteps, interv=0):
        nmon = sum(1 for it in range(iter0, iter0 + nsteps) if it % interv == 0) if interv > 0 else 0
        log = np.zeros(max(nmon, 1))
        self._check(lib().imexlb_step(self.h, iter0, nsteps, interv, _p(log, C.c_double)))
        return log[:nmon]

    def observe(self):
        """(momentum-exchange force on the obstacle, mass deviation sum(f))."""
        F = np.zeros(3)
        m = C.c_double()
        self._check(lib().imexlb_observe(self.h, _p(F, C.c_double), C.byref(m)))
        return F[:self.dim], m.value

    def step_observed(self, iter0, nsteps, interv, every):
        """step() that also returns the obstacle force after each iteration
        with iter % every == 0, shape (samples, dim)."""
        nmon = sum(1 for it in range(iter0, iter0 + nsteps) if it % interv == 0) if interv > 0 else 0
        nobs = sum(1 for it in range(iter0, iter0 + nsteps) if it % every == 0) if every > 0 else 0
        log = np.zeros(max(nmon, 1))
        F = np.zeros(max(nobs * self.dim, 1))
        self._check(lib().imexlb_step_observed(self.h, iter0, nsteps, interv, _p(log, C.c_double),
                                               every, _p(F, C.c_double)))
        return log[:nmon], F[:nobs * self.dim].reshape(nobs, self.dim)

    def download(self, f=True, fb=True, p=True, u=True):
        n = self.n
        outs = [np.empty(n * self.nq) if f else None, np.empty(n * self.nq) if fb else None,
                np.empty(n) if p else None, np.empty(n * self.dim) if u else None]
        self._check(lib().imexlb_download(self.h, *[_p(o, C.c_double) for o in outs]))
        return tuple(outs)

    def download_ptr(self, f, fb, p, u):
        cast = lambda x: C.cast(x, _pd) if x else None
        self._check(lib().imexlb_download(self.h, cast(f), cast(fb), cast(p), cast(u)))

    def info(self):
        i = Info()
        self._check(lib().imexlb_get_info(self.h, C.byref(i)))
        return i

    def profile_reset(self, timing=False):
        self._check(lib().imexlb_profile_reset(self.h, 1 if timing else 0))

    def profile(self):
        pr = Profile()
        self._check(lib().imexlb_profile_read(self.h, C.byref(pr)))
        return {"launches": list(pr.launches), "ms": list(pr.ms)}

    def sample(self, W, H):
        """(fluid fraction, p, ux, uy) at W x H pixel centres, shape (4, H, W)."""
        out = np.empty(4 * W * H, dtype=np.float32)
        self._check(lib().imexlb_sample(self.h, W, H, out.ctypes.data_as(C.POINTER(C.c_float))))
        return out.reshape(4, H, W)

    def init_state(self, rv=None):
        """The initial state on the device: InitUP with the 100 draws rv (or
        the rest state when rv is None), f = fb = 0; then init_pdf()."""
        r = None if rv is None else _f64(rv)
        self._check(lib().imexlb_init_state(self.h, _p(r, C.c_double)))

    def set_fp64_split(self, split):
        """Step-kernel variant of the FP64 path (share of FP64 operations in
        integer emulation; identical results for every variant)."""
        self._check(lib().imexlb_set_fp64_split(self.h, int(split)))

    def set_staged_kernel(self, on):
        """BF16 / FP16 storage on D3Q27: the step kernel that stages tiles in
        shared memory with bulk copies (True, the default) or the one that
        loads every population into registers (False); identical results."""
        self._check(lib().imexlb_testing_set_staged_kernel(self.h, 1 if on else 0))

    def set_fill_mode(self, mode):
        """Boundary copies inside the step kernel (FILL_FUSED, the default) or
        in a separate kernel after each step (FILL_KERNEL); identical results."""
        self._check(lib().imexlb_set_fill_mode(self.h, int(mode)))

    def set_watchdog(self, on=True):
        """step() raises ImexlbError (code ERR_DIVERGED) when a Monitor value
        of the call is NaN or infinite."""
        self._check(lib().imexlb_set_watchdog(self.h, 1 if on else 0))

    def fill_mode(self):
        m = _c_int()
        self._check(lib().imexlb_get_fill_mode(self.h, C.byref(m)))
        return m.value

    def stream(self):
        s = C.c_void_p()
        self._check(lib().imexlb_get_stream(self.h, C.byref(s)))
        return s.value

    def close(self):
        if getattr(self, "h", None):
            lib().imexlb_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Group:
    """The ranks of a multi-rank run (Solver handles made from
    rank_config / GroupSetup, in MPI rank order) stepped together with
    PassF across ranks (imexlb_group_*)."""

    def __init__(self, solvers):
        self.solvers = list(solvers)
        arr = (C.c_void_p * len(self.solvers))(*[s.h.value for s in self.solvers])
        g = C.c_void_p()
        rc = lib().imexlb_group_create(C.byref(g), arr, len(self.solvers))
        if rc != IMEXLB_OK:
            raise ImexlbError(rc, lib().imexlb_last_error(None).decode())
        self.g = g

    def step(self, iter0, nsteps, interv=0):
        nmon = sum(1 for it in range(iter0, iter0 + nsteps) if interv > 0 and it % interv == 0)
        log = np.zeros(max(nmon, 1))
        rc = lib().imexlb_group_step(self.g, iter0, nsteps, interv, _p(log, C.c_double))
        if rc != IMEXLB_OK:
            raise ImexlbError(rc, lib().imexlb_group_last_error(self.g).decode())
        return log[:nmon]

    def close(self):
        if getattr(self, "g", None):
            lib().imexlb_group_destroy(self.g)
            self.g = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Lockstep stepping of many Solver handles (same device, dimension and
    reduced-precision storage, each stepped at least once)."""

    def __init__(self, solvers):
        self.solvers = list(solvers)
        arr = (C.c_void_p * len(self.solvers))(*[s.h.value for s in self.solvers])
        b = C.c_void_p()
        rc = lib().imexlb_batch_create(C.byref(b), arr, len(self.solvers))
        if rc != IMEXLB_OK:
            raise ImexlbError(rc, "imexlb_batch_create failed")
        self.b = b

    def _check(self, rc):
        if rc != IMEXLB_OK:
            raise ImexlbError(rc, lib().imexlb_batch_last_error(self.b).decode())

    def set_mode(self, mode):
        """BATCH_LOCKSTEP (one launch per iteration, graph-replayed) or
        BATCH_PERSISTENT (one cooperative launch per call)."""
        self._check(lib().imexlb_batch_set_mode(self.b, int(mode)))

    def tune(self, trial=4):
        sh = C.c_int()
        self._check(lib().imexlb_batch_tune(self.b, trial, C.byref(sh)))
        return sh.value

    def step(self, nsteps=0, steps=None):
        if steps is None:
            self._check(lib().imexlb_batch_step(self.b, nsteps, None))
        else:
            st = _i32(steps)
            self._check(lib().imexlb_batch_step(self.b, 0, _p(st, C.c_int)))

    def close(self):
        if getattr(self, "b", None):
            lib().imexlb_batch_destroy(self.b)
            self.b = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
