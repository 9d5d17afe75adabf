"""ctypes binding of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Loaded by tests/, __graft_entry__.smoke() and bench.py's CPU legs.  The
oracle's config struct has the layout of the C ABI's b2d_config, so the
product's ctypes struct is passed through unchanged.
"""
import ctypes
import os

import numpy as np

from . import build as _build

c_int32 = ctypes.c_int32
c_double = ctypes.c_double
c_dp = ctypes.POINTER(ctypes.c_double)


class OracleError(ctypes.Structure):
    _fields_ = [
        ("code", c_int32), ("run", c_int32), ("block_i", c_int32), ("block_j", c_int32),
        ("zone_i", c_int32), ("zone_j", c_int32), ("value", c_double), ("x", c_double),
        ("y", c_double), ("time", c_double), ("binary", c_double * 4),
    ]


class PointMass(ctypes.Structure):
    _fields_ = [("m", c_double), ("x", c_double), ("y", c_double), ("vx", c_double), ("vy", c_double)]


_lib = None


def load():
    global _lib
    if _lib is None:
        path = _build.build()
        lib = ctypes.CDLL(path)
        vp = ctypes.c_void_p
        lib.oracle_advance.restype = c_int32
        lib.oracle_advance.argtypes = [vp, c_dp, c_dp, c_dp, c_dp, ctypes.POINTER(ctypes.c_int64), c_int32, c_dp,
                                       c_int32, ctypes.POINTER(OracleError), c_dp, ctypes.c_int64, c_dp]
        lib.oracle_max_signal_speed.restype = c_double
        lib.oracle_max_signal_speed.argtypes = [vp, c_dp]
        lib.oracle_max_signal_speed_rows.restype = c_double
        lib.oracle_max_signal_speed_rows.argtypes = [vp, c_dp, c_int32, c_int32]
        lib.oracle_stage_rows.restype = c_int32
        lib.oracle_stage_rows.argtypes = [vp, c_dp, c_dp, c_dp, c_double, c_dp, c_dp, c_dp, c_dp, c_double,
                                          c_double, c_int32, c_int32, ctypes.POINTER(OracleError)]
        lib.oracle_initial_state.restype = c_int32
        lib.oracle_initial_state.argtypes = [vp, vp, c_dp]
        lib.oracle_orbital_state.restype = None
        lib.oracle_orbital_state.argtypes = [vp, c_double, ctypes.POINTER(PointMass), ctypes.POINTER(PointMass)]
        lib.oracle_plm_gradient.restype = c_double
        lib.oracle_plm_gradient.argtypes = [c_double, c_double, c_double, c_double]
        lib.oracle_hlle.restype = None
        lib.oracle_hlle.argtypes = [vp, c_dp, c_dp, c_int32, c_double, c_dp]
        lib.oracle_physical_flux.restype = None
        lib.oracle_physical_flux.argtypes = [vp, c_dp, c_int32, c_double, c_dp]
        lib.oracle_prim_to_cons.restype = None
        lib.oracle_prim_to_cons.argtypes = [vp, c_dp, c_dp]
        lib.oracle_cons_to_prim.restype = c_int32
        lib.oracle_cons_to_prim.argtypes = [vp, c_dp, c_dp]
        lib.oracle_source_terms.restype = None
        lib.oracle_source_terms.argtypes = [vp, c_dp, c_dp, c_double, c_double, c_double, c_double, c_dp]
        lib.oracle_cell_centers.restype = None
        lib.oracle_cell_centers.argtypes = [vp, c_int32, c_dp]
        lib.oracle_block_vertices.restype = None
        lib.oracle_block_vertices.argtypes = [vp, c_int32, c_dp]
        _lib = lib
    return _lib


def _dp(a):
    return a.ctypes.data_as(c_dp)


class OracleHydroError(RuntimeError):
    def __init__(self, err):
        self.err = err
        super().__init__("oracle hydro error %d value %g at (%g, %g)" % (err.code, err.value, err.x, err.y))


class OracleState:
    """State (src/state.rs:57-62) held by the oracle: conserved in block layout,
    per-block ledger, per-block orbital-element change, time, iteration."""

    def __init__(self, cfg, cons, background=None, ledger=None, time=0.0, iteration=0, elements=None):
        self.cfg = cfg
        self.cons = np.array(cons, dtype=np.float64, copy=True)
        self.background = self.cons.copy() if background is None else np.ascontiguousarray(background, np.float64)
        nb = cfg.num_blocks
        nf = self.cons.shape[-1]
        self.ledger = np.zeros((nb, nb, 7, nf)) if ledger is None else np.array(ledger, dtype=np.float64)
        self.elements = np.zeros((nb, nb, 7, 4)) if elements is None else np.array(elements, dtype=np.float64)
        self.time = ctypes.c_double(time)
        self.iteration = ctypes.c_int64(iteration)
        self.tracers = None

    def set_tracers(self, xy):
        self.tracers = np.array(xy, dtype=np.float64).reshape(-1, 2).copy()

    def advance(self, fold, nthreads=None):
        lib = load()
        if nthreads is None:
            nthreads = 2 * (os.cpu_count() or 1)
        dt = ctypes.c_double(0)
        err = OracleError()
        tr = self.tracers
        rc = lib.oracle_advance(ctypes.byref(self.cfg), _dp(self.cons), _dp(self.ledger), _dp(self.background),
                                ctypes.byref(self.time), ctypes.byref(self.iteration), int(fold), ctypes.byref(dt),
                                int(nthreads), ctypes.byref(err), None if tr is None else _dp(tr),
                                0 if tr is None else len(tr), _dp(self.elements))
        if rc:
            raise OracleHydroError(err)
        return dt.value


def initial_state(cfg, model_struct, shape):
    out = np.empty(shape, dtype=np.float64)
    load().oracle_initial_state(ctypes.byref(cfg), ctypes.byref(model_struct), _dp(out))
    return out


def disk_initial_state(mesh, hydro, physics, model, run=0):
    """The oracle's initial state of a run described by the host package's
    Mesh / hydro / Physics / DiskModel (BlockState::from_model,
    src/state.rs:74-86, plus the synthetic cavity and noise), without loading
    the product library.  Returns (state in block layout, oracle config)."""
    from binary2d.config import to_c
    from binary2d.scheme import disk_model_struct, state_shape
    cfg = to_c(mesh, hydro, physics)
    return initial_state(cfg, disk_model_struct(model, run), state_shape(mesh, hydro)), cfg


def max_signal_speed(cfg, cons):
    cons = np.ascontiguousarray(cons, np.float64)
    return load().oracle_max_signal_speed(ctypes.byref(cfg), _dp(cons))


def max_signal_speed_rows(cfg, cons, row_lo, row_hi):
    """The maximum signal speed over block rows [row_lo, row_hi) of cons."""
    return load().oracle_max_signal_speed_rows(ctypes.byref(cfg), _dp(cons), int(row_lo), int(row_hi))


def stage_rows(cfg, cons_in, cons_out, background, led_in, led_out, time, dt, row_lo, row_hi,
               base=None, led_base=None, bf=0.0):
    """One RK stage of the blocks in block rows [row_lo, row_hi) (a row slab):
    reads the slab and its 2-zone halo rows of cons_in, writes the slab of
    cons_out and led_out; with `base` the RK average with weight bf follows.
    Raises OracleHydroError on a failing zone of the slab."""
    err = OracleError()
    rc = load().oracle_stage_rows(ctypes.byref(cfg), _dp(cons_in), _dp(cons_out),
                                  None if base is None else _dp(base), float(bf), _dp(background), _dp(led_in),
                                  _dp(led_out), None if led_base is None else _dp(led_base), float(time), float(dt),
                                  int(row_lo), int(row_hi), ctypes.byref(err))
    if rc:
        raise OracleHydroError(err)


def orbital_state(cfg, t):
    p1, p2 = PointMass(), PointMass()
    load().oracle_orbital_state(ctypes.byref(cfg), t, ctypes.byref(p1), ctypes.byref(p2))
    return p1, p2
