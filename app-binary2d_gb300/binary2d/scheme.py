"""Host mirror of scheme::advance (src/scheme.rs:323-349) over the C ABI.

A `Runtime` owns a b2d context: the device copy of one or more runs' State
and BlockData.  `Runtime.advance(fold)` is scheme::advance: one dt from the
max signal speed, then `fold` Runge–Kutta steps, raising HydroError (the
reference's Err(HydroError), src/physics.rs:47-71) and leaving the state as
it was when a zone fails.
"""
import ctypes
from dataclasses import dataclass
from typing import List, Optional, Sequence, Tuple

import numpy as np

from . import _lib
from ._lib import B2DConfig, B2DDiskModel, B2DError
from .config import DiskModel, Euler, Isothermal, Mesh, Physics, num_fields, to_c

PRECISIONS = {"fp64": 0, "fp32_state64": 1, "fp32_comp": 2}
ERROR_NAMES = {1: "NegativeDensity", 2: "NegativePressure", 3: "OrbitalEvolutionError",
               4: "Timeout", 5: "Cuda", 6: "Invalid", 7: "Unsupported"}
ITEMS = ("sink1", "sink2", "grav1", "grav2", "buffer", "cooling", "fake_mass")


class B2DException(RuntimeError):
    pass


class HydroError(B2DException):
    """A zone failed cons→prim: HydroErrorType::{NegativeDensity, NegativePressure}."""

    def __init__(self, err: B2DError):
        self.code = err.code
        self.kind = ERROR_NAMES.get(err.code, str(err.code))
        self.run = err.run
        self.block = (err.block_i, err.block_j)
        self.zone = (err.zone_i, err.zone_j)
        self.value = err.value
        self.position = (err.x, err.y)
        self.time = err.time
        self.binary = tuple(err.binary)
        super().__init__("%s %.4e at position (%.4f %.4f), when the binary was at (%.4f %.4f) (%.4f %.4f)"
                         % (self.kind, self.value, err.x, err.y, *self.binary))


def _check(status: int):
    if status != 0:
        raise B2DException("b2d error %d (%s): %s" % (status, ERROR_NAMES.get(status, "?"), _lib.last_error()))


def _dp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


@dataclass
class Run:
    mesh: Mesh
    hydro: object
    physics: Physics


def disk_model_struct(model: DiskModel, run: int = 0) -> B2DDiskModel:
    """The b2d_disk_model of `model` for run index `run` (plain data; building
    it loads no library)."""
    from .config import MODEL_KINDS
    m = B2DDiskModel()
    m.surface_density = model.surface_density
    m.mach_number = model.mach_number if model.mach_number is not None else 0.0
    m.cavity_radius = model.cavity_radius
    m.cavity_floor = model.cavity_floor
    m.noise = model.noise
    m.seed = model.seed
    m.run = run
    m.kind = MODEL_KINDS[model.kind]
    m.disk_mass = model.disk_mass
    m.disk_width = model.disk_width
    m.disk_radius = model.disk_radius
    m.disk_softening = model.softening_length
    m.core_radius = model.core_radius
    m.edge_width = model.edge_width
    return m


def state_shape(mesh: Mesh, hydro) -> Tuple[int, ...]:
    """Block layout [nb, nb, bs, bs, nf] of a run's conserved state."""
    return (mesh.num_blocks, mesh.num_blocks, mesh.block_size, mesh.block_size, num_fields(hydro))


def initial_state(mesh: Mesh, hydro, physics: Physics, model: DiskModel, run: int = 0) -> np.ndarray:
    """BlockState::from_model for the InfiniteDisk model plus the synthetic
    cavity/noise; returns the conserved state in block layout
    [nb, nb, bs, bs, nf]."""
    lib = _lib.load()
    c = to_c(mesh, hydro, physics)
    m = disk_model_struct(model, run)
    out = np.empty(state_shape(mesh, hydro), dtype=np.float64)
    _check(lib.b2d_initial_state(ctypes.byref(c), ctypes.byref(m), _dp(out)))
    return out


class Runtime:
    """A device context holding the state of `runs` (a list of Run)."""

    def __init__(self, runs: Sequence[Run], precision: str = "fp64"):
        self.lib = _lib.load()
        self.runs = list(runs)
        self.nf = num_fields(self.runs[0].hydro)
        arr = (B2DConfig * len(self.runs))(*[to_c(r.mesh, r.hydro, r.physics) for r in self.runs])
        self._cfgs = arr
        st = ctypes.c_int32(0)
        self.ctx = self.lib.b2d_create(arr, len(self.runs), PRECISIONS[precision], ctypes.byref(st))
        if not self.ctx:
            raise B2DException("b2d_create failed (%d): %s" % (st.value, _lib.last_error()))
        self.precision = precision

    def close(self):
        if getattr(self, "ctx", None):
            self.lib.b2d_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- state ---------------------------------------------------------------
    def upload(self, run: int, cons: np.ndarray, background: Optional[np.ndarray] = None,
               ledger: Optional[np.ndarray] = None, time: float = 0.0, iteration: int = 0):
        cons = np.ascontiguousarray(cons, dtype=np.float64)
        bg = cons if background is None else np.ascontiguousarray(background, dtype=np.float64)
        led = None if ledger is None else np.ascontiguousarray(ledger, dtype=np.float64)
        _check(self.lib.b2d_upload_state(self.ctx, run, _dp(cons), _dp(bg), None if led is None else _dp(led),
                                         time, int(iteration), 1))

    def upload_conserved(self, run: int, cons: np.ndarray):
        cons = np.ascontiguousarray(cons, dtype=np.float64)
        _check(self.lib.b2d_upload_conserved(self.ctx, run, _dp(cons)))

    def upload_conserved_async(self, run: int, cons: np.ndarray):
        """Queue an upload of `cons` (contiguous float64, ideally pinned); it
        must stay unchanged until a later download has landed."""
        assert cons.flags.c_contiguous and cons.dtype == np.float64
        _check(self.lib.b2d_upload_conserved_async(self.ctx, run, _dp(cons)))

    def download_async(self, run: int, out: np.ndarray):
        """Queue a download of the state (as queued so far) into `out`."""
        assert out.flags.c_contiguous and out.dtype == np.float64
        _check(self.lib.b2d_download_async(self.ctx, run, _dp(out)))

    def transfers_wait(self, pending: int = 0):
        """Block until every transfer (pending=0) or every download but the
        newest (pending=1) has landed."""
        _check(self.lib.b2d_transfers_wait(self.ctx, int(pending)))

    def download(self, run: int = 0, out: Optional[np.ndarray] = None) -> Tuple[np.ndarray, float, int]:
        m = self.runs[run].mesh
        if out is None:
            out = np.empty((m.num_blocks, m.num_blocks, m.block_size, m.block_size, self.nf), dtype=np.float64)
        t = ctypes.c_double(0)
        num, den = ctypes.c_int64(0), ctypes.c_int64(0)
        _check(self.lib.b2d_download_state(self.ctx, run, _dp(out), ctypes.byref(t), ctypes.byref(num),
                                           ctypes.byref(den)))
        return out, t.value, num.value

    def time(self, run: int = 0) -> Tuple[float, int]:
        t = ctypes.c_double(0)
        num, den = ctypes.c_int64(0), ctypes.c_int64(0)
        _check(self.lib.b2d_download_state(self.ctx, run, None, ctypes.byref(t), ctypes.byref(num),
                                           ctypes.byref(den)))
        return t.value, num.value

    def ledger(self, run: int = 0) -> np.ndarray:
        """Per-block integrated_source_terms [nb, nb, 7, nf] (state.rs:44-49)."""
        m = self.runs[run].mesh
        out = np.empty((m.num_blocks, m.num_blocks, 7, self.nf), dtype=np.float64)
        _check(self.lib.b2d_download_ledger(self.ctx, run, _dp(out)))
        return out

    def elements(self, run: int = 0) -> np.ndarray:
        """Per-block orbital_elements_change [nb, nb, 7, 4] of (a, M, q, e)."""
        m = self.runs[run].mesh
        out = np.empty((m.num_blocks, m.num_blocks, 7, 4), dtype=np.float64)
        _check(self.lib.b2d_download_elements(self.ctx, run, _dp(out)))
        return out

    def upload_elements(self, run: int, elements: np.ndarray):
        e = np.ascontiguousarray(elements, dtype=np.float64)
        _check(self.lib.b2d_upload_elements(self.ctx, run, _dp(e)))

    def set_tracers(self, run: int, xy: np.ndarray):
        """Massless tracers of a run: `xy` of shape [n, 2]."""
        xy = np.ascontiguousarray(xy, dtype=np.float64).reshape(-1, 2)
        self._ntracers = getattr(self, "_ntracers", {})
        self._ntracers[run] = len(xy)
        _check(self.lib.b2d_set_tracers(self.ctx, run, len(xy), _dp(xy) if len(xy) else None))

    def tracers(self, run: int = 0) -> np.ndarray:
        n = getattr(self, "_ntracers", {}).get(run, 0)
        out = np.empty((n, 2), dtype=np.float64)
        if n:
            _check(self.lib.b2d_get_tracers(self.ctx, run, _dp(out)))
        return out

    def max_signal_speed(self, run: int = 0) -> float:
        v = ctypes.c_double(0)
        _check(self.lib.b2d_max_signal_speed(self.ctx, run, ctypes.byref(v)))
        return v.value

    # -- the step --------------------------------------------------------------
    def advance(self, fold: int) -> np.ndarray:
        """scheme::advance for every run; returns the dt of each run."""
        dts = np.zeros(len(self.runs), dtype=np.float64)
        err = B2DError()
        st = self.lib.b2d_advance(self.ctx, int(fold), _dp(dts), ctypes.byref(err))
        if st in (1, 2, 3):
            raise HydroError(err)
        _check(st)
        return dts

    def advance_async(self, fold: int):
        _check(self.lib.b2d_advance_async(self.ctx, int(fold)))

    def synchronize(self) -> np.ndarray:
        dts = np.zeros(len(self.runs), dtype=np.float64)
        err = B2DError()
        st = self.lib.b2d_synchronize(self.ctx, _dp(dts), ctypes.byref(err))
        if st in (1, 2, 3):
            raise HydroError(err)
        _check(st)
        return dts

    # -- row slabs (one run split across contexts) ------------------------------
    def set_slab(self, run: int, block_row_lo: int, block_row_hi: int):
        """Make block rows [lo, hi) of `run` this context's slab ((0, 0): the
        whole run).  A slab's stage launches cover its block-aligned tiles of
        the tile height (row chunks apply to whole runs only)."""
        _check(self.lib.b2d_set_slab(self.ctx, run, int(block_row_lo), int(block_row_hi)))

    def slab_begin(self, fold: int, amax):
        """Start an advance whose dt comes from amax (one global maximum signal
        speed per run, the max over all slabs)."""
        a = np.ascontiguousarray(np.atleast_1d(np.asarray(amax, dtype=np.float64)))
        _check(self.lib.b2d_slab_begin(self.ctx, int(fold), _dp(a)))

    def slab_stage(self):
        _check(self.lib.b2d_slab_stage(self.ctx))

    def slab_end(self) -> np.ndarray:
        dts = np.zeros(len(self.runs), dtype=np.float64)
        err = B2DError()
        st = self.lib.b2d_slab_end(self.ctx, _dp(dts), ctypes.byref(err))
        if st in (1, 2, 3):
            raise HydroError(err)
        _check(st)
        return dts

    def slab_rows(self, run: int, row0: int, nrows: int) -> np.ndarray:
        """Zone rows [row0, row0 + nrows) (periodic) of the next stage's input,
        as stored: [nf, nrows, N] FP64, or for the compensated FP32 state
        [nf, 2, nrows, N] FP32 (hi and lo words)."""
        N = self.runs[run].mesh.zones_per_side()
        if self.precision == "fp32_comp":
            out = np.empty((self.nf, 2, nrows, N), dtype=np.float32)
        else:
            out = np.empty((self.nf, nrows, N), dtype=np.float64)
        _check(self.lib.b2d_slab_rows(self.ctx, run, int(row0), int(nrows), out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 0))
        return out

    def put_slab_rows(self, run: int, row0: int, rows: np.ndarray):
        """Write rows got from slab_rows of a context of the same precision."""
        dtype = np.float32 if self.precision == "fp32_comp" else np.float64
        r = np.ascontiguousarray(rows, dtype=dtype)
        _check(self.lib.b2d_slab_rows(self.ctx, run, int(row0), r.shape[-2], r.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 1))

    # -- tuning / introspection ----------------------------------------------
    def set_tile(self, w: int = 0, h: int = 0):
        _check(self.lib.b2d_set_tile(self.ctx, w, h))

    def tile(self) -> Tuple[int, int]:
        w, h = ctypes.c_int32(0), ctypes.c_int32(0)
        _check(self.lib.b2d_get_tile(self.ctx, ctypes.byref(w), ctypes.byref(h)))
        return w.value, h.value

    def set_strip_rows(self, rows: int = 0):
        """Row chunks of at most `rows` rows, crossing block boundaries, for the
        paired FP32 kernel (0: block-aligned tiles of the tile height)."""
        _check(self.lib.b2d_set_strip_rows(self.ctx, int(rows)))

    def strip_rows(self) -> int:
        r = ctypes.c_int32(0)
        _check(self.lib.b2d_get_strip_rows(self.ctx, ctypes.byref(r)))
        return r.value

    def autotune(self, fold: int = 2, reps: int = 2):
        """Pick the fastest tile shape for this context; returns (w, h, ms/stage)."""
        w, h, ms = ctypes.c_int32(0), ctypes.c_int32(0), ctypes.c_double(0)
        _check(self.lib.b2d_autotune(self.ctx, fold, reps, ctypes.byref(w), ctypes.byref(h), ctypes.byref(ms)))
        return w.value, h.value, ms.value

    def set_graphs(self, on: bool):
        _check(self.lib.b2d_set_graphs(self.ctx, int(bool(on))))

    def launch_count(self) -> int:
        return int(self.lib.b2d_launch_count(self.ctx))

    def launches_per_advance(self, fold: int) -> int:
        return int(self.lib.b2d_launches_per_advance(self.ctx, fold))

    def set_instrument(self, on: bool):
        _check(self.lib.b2d_set_instrument(self.ctx, int(bool(on))))

    def stage_stats(self) -> Tuple[int, float]:
        n, ms = ctypes.c_int64(0), ctypes.c_double(0)
        _check(self.lib.b2d_stage_stats(self.ctx, ctypes.byref(n), ctypes.byref(ms)))
        return n.value, ms.value

    def time_stages(self, fold: int, reps: int) -> float:
        v = ctypes.c_double(0)
        _check(self.lib.b2d_time_stages(self.ctx, fold, reps, ctypes.byref(v)))
        return v.value

    def stream(self) -> int:
        s = ctypes.c_void_p(0)
        _check(self.lib.b2d_stream(self.ctx, ctypes.byref(s)))
        return s.value or 0


def set_device(device: int):
    """Select the CUDA device of the calling thread inside libb2d."""
    _check(_lib.load().b2d_set_device(int(device)))


def pin(array: np.ndarray):
    """Page-lock a host array for asynchronous copies (cudaHostRegister)."""
    _check(_lib.load().b2d_pin_host(array.ctypes.data, array.nbytes))


def unpin(array: np.ndarray):
    _check(_lib.load().b2d_unpin_host(array.ctypes.data))
