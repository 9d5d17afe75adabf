"""ctypes binding of libb2d.so (the C ABI declared in include/b2d.h).

The library is built in-tree (app-binary2d_gb300/_build/libb2d.so).  Loading
fails loudly when it is missing: there is no CPU fallback.
"""
import ctypes
import os

_PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(_PKG, "_build", "libb2d.so")

c_int32 = ctypes.c_int32
c_int64 = ctypes.c_int64
c_double = ctypes.c_double
c_dp = ctypes.POINTER(ctypes.c_double)


class B2DConfig(ctypes.Structure):
    """b2d_config: Mesh + hydro + Physics, flattened (include/b2d.h)."""
    _fields_ = [
        ("num_blocks", c_int32), ("block_size", c_int32), ("domain_radius", c_double),
        ("hydro_kind", c_int32), ("density_index", c_int32),
        ("mach_number", c_double), ("gamma_law_index", c_double), ("cooling_coefficient", c_double),
        ("pressure_floor", c_double), ("density_floor", c_double),
        ("has_pressure_floor", c_int32), ("has_density_floor", c_int32),
        ("cooling_slow_start", c_int32), ("cooling_kind", c_int32), ("cooling_beta", c_double),
        ("buffer_rate", c_double), ("buffer_scale", c_double), ("binary_eccentricity", c_double),
        ("binary_mass_ratio", c_double), ("lambda_multiplier", c_double), ("viscosity", c_double),
        ("viscosity_kind", c_int32), ("sink_model", c_int32),
        ("cfl", c_double), ("plm", c_double), ("plm_density_trigger", c_double),
        ("fake_mass_threshold", c_double), ("fake_mass_rate", c_double), ("mach_ceiling", c_double),
        ("sink_radius", c_double), ("sink_rate", c_double), ("softening_length", c_double),
        ("dt_min", c_double),
        ("has_plm_density_trigger", c_int32), ("one_body", c_int32), ("rk_order", c_int32),
        ("has_mach_ceiling", c_int32), ("has_softening_length", c_int32), ("has_dt_min", c_int32),
    ]


class B2DError(ctypes.Structure):
    """b2d_error: HydroError (src/physics.rs:47-71) as plain data."""
    _fields_ = [
        ("code", c_int32), ("run", c_int32), ("block_i", c_int32), ("block_j", c_int32),
        ("zone_i", c_int32), ("zone_j", c_int32), ("value", c_double), ("x", c_double),
        ("y", c_double), ("time", c_double), ("binary", c_double * 4),
    ]


class B2DDiskModel(ctypes.Structure):
    _fields_ = [
        ("surface_density", c_double), ("mach_number", c_double), ("cavity_radius", c_double),
        ("cavity_floor", c_double), ("noise", c_double), ("seed", ctypes.c_uint64),
        ("run", c_int32), ("kind", c_int32), ("disk_mass", c_double), ("disk_width", c_double),
        ("disk_radius", c_double), ("disk_softening", c_double), ("core_radius", c_double),
        ("edge_width", c_double),
    ]


_lib = None

# (name, restype, argtypes)
_SIGNATURES = [
    ("b2d_create", ctypes.c_void_p, [ctypes.POINTER(B2DConfig), c_int32, c_int32, ctypes.POINTER(c_int32)]),
    ("b2d_destroy", None, [ctypes.c_void_p]),
    ("b2d_last_error", ctypes.c_char_p, []),
    ("b2d_num_fields", c_int32, [ctypes.c_void_p]),
    ("b2d_upload_state", c_int32, [ctypes.c_void_p, c_int32, c_dp, c_dp, c_dp, c_double, c_int64, c_int64]),
    ("b2d_upload_conserved", c_int32, [ctypes.c_void_p, c_int32, c_dp]),
    ("b2d_download_state", c_int32, [ctypes.c_void_p, c_int32, c_dp, c_dp,
                                     ctypes.POINTER(c_int64), ctypes.POINTER(c_int64)]),
    ("b2d_download_ledger", c_int32, [ctypes.c_void_p, c_int32, c_dp]),
    ("b2d_advance", c_int32, [ctypes.c_void_p, c_int32, c_dp, ctypes.POINTER(B2DError)]),
    ("b2d_advance_async", c_int32, [ctypes.c_void_p, c_int32]),
    ("b2d_synchronize", c_int32, [ctypes.c_void_p, c_dp, ctypes.POINTER(B2DError)]),
    ("b2d_max_signal_speed", c_int32, [ctypes.c_void_p, c_int32, c_dp]),
    ("b2d_initial_state", c_int32, [ctypes.POINTER(B2DConfig), ctypes.POINTER(B2DDiskModel), c_dp]),
    ("b2d_set_tile", c_int32, [ctypes.c_void_p, c_int32, c_int32]),
    ("b2d_set_strip_rows", c_int32, [ctypes.c_void_p, c_int32]),
    ("b2d_get_strip_rows", c_int32, [ctypes.c_void_p, ctypes.POINTER(c_int32)]),
    ("b2d_get_tile", c_int32, [ctypes.c_void_p, ctypes.POINTER(c_int32), ctypes.POINTER(c_int32)]),
    ("b2d_set_graphs", c_int32, [ctypes.c_void_p, c_int32]),
    ("b2d_launch_count", c_int64, [ctypes.c_void_p]),
    ("b2d_launches_per_advance", c_int64, [ctypes.c_void_p, c_int32]),
    ("b2d_time_stages", c_int32, [ctypes.c_void_p, c_int32, c_int32, c_dp]),
    ("b2d_set_instrument", c_int32, [ctypes.c_void_p, c_int32]),
    ("b2d_stage_stats", c_int32, [ctypes.c_void_p, ctypes.POINTER(c_int64), c_dp]),
    ("b2d_stream", c_int32, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]),
    ("b2d_pin_host", c_int32, [ctypes.c_void_p, ctypes.c_uint64]),
    ("b2d_unpin_host", c_int32, [ctypes.c_void_p]),
    ("b2d_set_device", c_int32, [c_int32]),
    ("b2d_download_elements", c_int32, [ctypes.c_void_p, c_int32, c_dp]),
    ("b2d_upload_conserved_async", c_int32, [ctypes.c_void_p, c_int32, c_dp]),
    ("b2d_download_async", c_int32, [ctypes.c_void_p, c_int32, c_dp]),
    ("b2d_transfers_wait", c_int32, [ctypes.c_void_p, c_int32]),
    ("b2d_upload_elements", c_int32, [ctypes.c_void_p, c_int32, c_dp]),
    ("b2d_set_tracers", c_int32, [ctypes.c_void_p, c_int32, c_int64, c_dp]),
    ("b2d_get_tracers", c_int32, [ctypes.c_void_p, c_int32, c_dp]),
    ("b2d_stage_noalloc", c_int32, [ctypes.POINTER(B2DConfig), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                    ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, c_double,
                                    c_double, c_double, ctypes.c_void_p, ctypes.POINTER(B2DError), ctypes.c_void_p]),
    ("b2d_set_slab", c_int32, [ctypes.c_void_p, c_int32, c_int32, c_int32]),
    ("b2d_slab_begin", c_int32, [ctypes.c_void_p, c_int32, c_dp]),
    ("b2d_slab_stage", c_int32, [ctypes.c_void_p]),
    ("b2d_slab_end", c_int32, [ctypes.c_void_p, c_dp, ctypes.POINTER(B2DError)]),
    ("b2d_slab_rows", c_int32, [ctypes.c_void_p, c_int32, c_int32, c_int32, c_dp, c_int32]),
    ("b2d_autotune", c_int32, [ctypes.c_void_p, c_int32, c_int32, ctypes.POINTER(c_int32), ctypes.POINTER(c_int32), c_dp]),
]

EXPORTED = [name for name, _, _ in _SIGNATURES]


def load(path: str = LIB_PATH):
    """Load libb2d.so and attach argument types.  Raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(
            "libb2d.so not found at %s: build it with `python -c \"import __graft_entry__ as g; g.build()\"` "
            "(there is no CPU fallback)" % path)
    lib = ctypes.CDLL(path)
    for name, res, args in _SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def last_error() -> str:
    return load().b2d_last_error().decode()
