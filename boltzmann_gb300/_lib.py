"""ctypes binding of libbz.so, the sm_103a kernels behind include/bz.h.

There is no fallback: if the library is missing or cannot be loaded, every call
raises ``BzLibraryError``. Build it with ``python -m boltzmann_gb300.build``.
"""
from __future__ import annotations

import ctypes
import os

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libbz.so")

BZ_OK, BZ_ERR_ARG, BZ_ERR_CUDA, BZ_ERR_WORKSPACE, BZ_ERR_UNSUPPORTED, BZ_ERR_TOO_LARGE = 0, 1, 2, 3, 4, 5
DEV_CAPACITY, DEV_LOOKBACK, DEV_NONFINITE, DEV_BINRANGE = 0x1, 0x2, 0x4, 0x8
QUIRK_SPLIT_WRAP, QUIRK_DEAD_IONFLAG, QUIRK_TRIGGER_LAST, FIX_MERGE_ENERGY = 0x1, 0x2, 0x4, 0x8
PER_KEY_TARGETS, MOMENT_EXCITATION, CLEAR_MOMENTS, RESAMPLE_IN_PLACE = 0x10, 0x20, 0x40, 0x80
ADVECT_NONE, ADVECT_1D, ADVECT_ENSEMBLE = 0, 1, 2
XS_TABLE, XS_REF_FITS = 0, 1
COLL_DIRECT, COLL_NULL = 0, 1

_ERRNAMES = {1: "invalid argument", 2: "CUDA error", 3: "workspace too small", 4: "unsupported configuration",
             5: "input larger than the entry point's fixed limit"}


class BzLibraryError(RuntimeError):
    pass


class BzError(RuntimeError):
    def __init__(self, fn, code):
        super().__init__(f"{fn} failed: {_ERRNAMES.get(code, code)} (status {code})")
        self.code = code


class BzParams(ctypes.Structure):
    _fields_ = [
        ("n_faces", ctypes.c_int32), ("n_nodes", ctypes.c_int32), ("bnf", ctypes.c_int32),
        ("advect", ctypes.c_int32), ("L", ctypes.c_double), ("dx", ctypes.c_double),
        ("dt", ctypes.c_double), ("nn", ctypes.c_double), ("gas_sigma", ctypes.c_double),
        ("e_exc", ctypes.c_double), ("nu_max", ctypes.c_double),
        ("xs_mode", ctypes.c_int32), ("coll_model", ctypes.c_int32), ("xs_n", ctypes.c_int32),
        ("flags", ctypes.c_int32), ("xs_emin", ctypes.c_double), ("xs_emax", ctypes.c_double),
        ("xs_table", ctypes.c_void_p), ("seed", ctypes.c_uint64), ("step", ctypes.c_uint64),
        ("step_ptr", ctypes.c_void_p),
    ]


class Particles(ctypes.Structure):
    """bz_particles_f32 / bz_particles_f64: five device pointers."""
    _fields_ = [("x", ctypes.c_void_p), ("vx", ctypes.c_void_p), ("vy", ctypes.c_void_p),
                ("vz", ctypes.c_void_p), ("w", ctypes.c_void_p)]


class Segments(ctypes.Structure):
    """bz_segments_f32 / bz_segments_f64: five device pointers, counts, nseg, half."""
    _fields_ = [("x", ctypes.c_void_p), ("vx", ctypes.c_void_p), ("vy", ctypes.c_void_p),
                ("vz", ctypes.c_void_p), ("w", ctypes.c_void_p), ("counts", ctypes.c_void_p),
                ("nseg", ctypes.c_int32), ("half", ctypes.c_int32)]


SEG_NEEDS_REPACK = 0x1
CONS_DIAG_STRIDE = 15  # float64 values per key of the resampling diagnostics

_lib = None

_vp = ctypes.c_void_p
_i32 = ctypes.c_int32
_i64 = ctypes.c_int64
_f64 = ctypes.c_double
_f32 = ctypes.c_float
_sz = ctypes.c_size_t
_P = ctypes.POINTER(BzParams)

_PROTOS = {
    "bz_version": (ctypes.c_char_p, []),
    "bz_push_workspace": (_sz, [_i64]),
    "bz_push_workspace_fast_f32": (_sz, [_i64, _i32]),
    "bz_push_workspace_fast_f64": (_sz, [_i64, _i32]),
    "bz_push_collide_f32": (ctypes.c_int, [_P, Particles, _vp, _i64, Particles, _i64, _vp, _vp, _vp, _vp, _vp, _vp,
                                           _sz, _vp, _vp]),
    "bz_push_collide_f64": (ctypes.c_int, [_P, Particles, _vp, _i64, Particles, _i64, _vp, _vp, _vp, _vp, _vp, _vp,
                                           _sz, _vp, _vp]),
    "bz_deposit_f32": (ctypes.c_int, [_P, Particles, _vp, _i64, _vp, _vp, _vp]),
    "bz_deposit_f64": (ctypes.c_int, [_P, Particles, _vp, _i64, _vp, _vp, _vp]),
    "bz_bin_workspace": (_sz, [_i64, _i32]),
    "bz_bin_f32": (ctypes.c_int, [_P, Particles, _vp, _i64, _i32, _vp, _f64, _vp, _vp, _vp, _vp, _vp, _sz, _vp, _vp]),
    "bz_bin_f64": (ctypes.c_int, [_P, Particles, _vp, _i64, _i32, _vp, _f64, _vp, _vp, _vp, _vp, _vp, _sz, _vp, _vp]),
    "bz_resample_workspace": (_sz, [_i64, _i32]),
    "bz_resample_f32": (ctypes.c_int, [_P, Particles, _vp, _i64, Particles, _vp, _i32, _vp, _vp, _f64, _f64, _f64,
                                       _f64, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _sz, _vp, _vp]),
    "bz_resample_f64": (ctypes.c_int, [_P, Particles, _vp, _i64, Particles, _vp, _i32, _vp, _vp, _f64, _f64, _f64,
                                       _f64, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _sz, _vp, _vp]),
    "bz_compact_workspace": (_sz, [_i64]),
    "bz_compact_f32": (ctypes.c_int, [Particles, _vp, _i64, Particles, _i64, _vp, _vp, _sz, _vp, _vp]),
    "bz_compact_f64": (ctypes.c_int, [Particles, _vp, _i64, Particles, _i64, _vp, _vp, _sz, _vp, _vp]),
    "bz_grid_update": (ctypes.c_int, [_i32, _vp, _vp, _vp, _vp, _vp]),
    "bz_ion_source_closure": (ctypes.c_int, [_i32, _vp, _vp, _vp]),
    "bz_ion_fluid": (ctypes.c_int, [_i32, _f64, _f64, _f64, _f64, _vp, _vp, _vp, _vp, _vp]),
    "bz_poisson_factor": (ctypes.c_int, [_i32, _f64, _vp, _vp, _vp]),
    "bz_field_step": (ctypes.c_int, [_i32, _f64, _f64, _f64, _f64, _f64, _f64, _f64, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                     _vp, _vp, _vp, _vp, _vp, _vp]),
    "bz_poisson": (ctypes.c_int, [_i32, _f64, _f64, _f64, _f64, _f64, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "bz_advance_clock": (ctypes.c_int, [_vp, _vp, _f64, _vp]),
    "bz_field_step_coop_workspace": (_sz, [_i32]),
    "bz_field_step_coop": (ctypes.c_int, [_i32, _f64, _f64, _f64, _f64, _f64, _f64, _f64, _vp, _vp, _vp, _vp, _vp, _vp,
                                          _vp, _vp, _vp, _vp, _vp, _vp, _vp, _sz, _vp]),
    "bz_field_step_select": (ctypes.c_int, [_i32]),
    "bz_philox4x32_10": (ctypes.c_int, [_vp, _vp, _i32, _i32, _vp, _vp]),
    "bz_field_step_selected": (ctypes.c_int, []),
    "bz_seg_push_workspace": (_sz, []),
    "bz_seg_push_workspace_nodes": (_sz, [_i32]),
    "bz_seg_push_shapes": (ctypes.c_int32, []),
    "bz_seg_push_shape_info": (ctypes.c_int, [ctypes.c_int32, _vp, _vp, _vp, _vp]),
    "bz_seg_push_select": (ctypes.c_int, [ctypes.c_int32]),
    "bz_seg_push_selected": (ctypes.c_int32, []),
    "bz_seg_push_collide_f32": (ctypes.c_int, [_P, Segments, Segments, _vp, _vp, _vp, _vp, _vp, _vp, _sz, _vp, _vp,
                                               _vp]),
    "bz_seg_push_collide_f64": (ctypes.c_int, [_P, Segments, Segments, _vp, _vp, _vp, _vp, _vp, _vp, _sz, _vp, _vp,
                                               _vp]),
    "bz_seg_repack_workspace": (_sz, [_i32]),
    "bz_seg_repack_f32": (ctypes.c_int, [ctypes.POINTER(Segments), Particles, _vp, _i64, Segments, _vp, _sz, _vp,
                                         _vp, _vp, _vp]),
    "bz_seg_repack_f64": (ctypes.c_int, [ctypes.POINTER(Segments), Particles, _vp, _i64, Segments, _vp, _sz, _vp,
                                         _vp, _vp, _vp]),
    "bz_seg_deposit_f32": (ctypes.c_int, [_P, Segments, _vp, _vp]),
    "bz_seg_deposit_f64": (ctypes.c_int, [_P, Segments, _vp, _vp]),
    "bz_seg_rebalance_f32": (ctypes.c_int, [Segments, Segments, _vp, _sz, _vp, _vp, _vp, _vp]),
    "bz_seg_rebalance_f64": (ctypes.c_int, [Segments, Segments, _vp, _sz, _vp, _vp, _vp, _vp]),
    "bz_seg_place_workspace": (_sz, [_i32]),
    "bz_seg_place_f32": (ctypes.c_int, [Segments, Particles, _vp, _i64, Segments, _vp, _sz, _vp, _vp, _vp]),
    "bz_seg_place_f64": (ctypes.c_int, [Segments, Particles, _vp, _i64, Segments, _vp, _sz, _vp, _vp, _vp]),
    "bz_seg_eedf_f32": (ctypes.c_int, [_P, Segments, ctypes.c_int32, ctypes.c_double, ctypes.c_double, _vp, _vp]),
    "bz_seg_eedf_f64": (ctypes.c_int, [_P, Segments, ctypes.c_int32, ctypes.c_double, ctypes.c_double, _vp, _vp]),
    "bz_seg_bin_workspace": (_sz, [_i32, _i64]),
    "bz_seg_bin_f32": (ctypes.c_int, [_P, Segments, _i32, _vp, _f64, _vp, _vp, _vp, _vp, _vp, _sz, _vp, _vp]),
    "bz_seg_bin_f64": (ctypes.c_int, [_P, Segments, _i32, _vp, _f64, _vp, _vp, _vp, _vp, _vp, _sz, _vp, _vp]),
    "bz_seg_bin_check_f32": (ctypes.c_int, [_P, Segments, _i32, _vp, _f64, _vp, _vp, _vp, _vp, _vp, _f64, _f64, _vp,
                                            _vp, _sz, _vp, _vp]),
    "bz_seg_bin_check_f64": (ctypes.c_int, [_P, Segments, _i32, _vp, _f64, _vp, _vp, _vp, _vp, _vp, _f64, _f64, _vp,
                                            _vp, _sz, _vp, _vp]),
    "bz_seg_resample_workspace": (_sz, [_i32, _i64, _i32]),
    "bz_seg_resample_f32": (ctypes.c_int, [_P, Segments, Particles, _i64, Segments, _i32, _vp, _vp, _f64, _f64, _f64,
                                           _f64, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _sz, _vp, _vp, _vp]),
    "bz_seg_resample_f64": (ctypes.c_int, [_P, Segments, Particles, _i64, Segments, _i32, _vp, _vp, _f64, _f64, _f64,
                                           _f64, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _sz, _vp, _vp, _vp]),
    "bz_push_collide_f32_noalloc": (ctypes.c_int, [_P, Particles, _vp, _i64, Particles, _i64, _vp, _vp, _vp, _vp,
                                                   _vp, _vp, _vp]),
    "bz_push_noalloc_scratch_address": (ctypes.c_int, [_vp]),
    "bz_set_wait_limit": (ctypes.c_int, [ctypes.c_uint32]),
    "bz_wait_limit": (ctypes.c_uint32, []),
    "bz_lookback_selftest_workspace": (_sz, [_i32]),
    "bz_lookback_selftest": (ctypes.c_int, [_i32, _i32, _vp, _vp, _sz, _vp, _vp]),
    "bz_mlp_wait_selftest": (ctypes.c_int, [_i32, _vp, _vp]),
    "bz_mlp_param_count": (ctypes.c_int32, []),
    "bz_mlp_select": (ctypes.c_int, [_i32]),
    "bz_mlp_selected": (ctypes.c_int32, []),
    "bz_mlp_status": (ctypes.c_int, [_vp]),
    "bz_mlp_sync": (ctypes.c_int, [_vp, _vp, _vp, _vp]),
    "bz_mlp_forward": (ctypes.c_int, [_vp, _vp, _vp, _vp, _i32, _vp, _vp, _vp]),
    "bz_mlp_backward_workspace": (_sz, [_i32]),
    "bz_mlp_backward": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _i32, _vp, _vp, _vp, _vp, _vp, _sz, _vp]),
    "bz_mlp_adam": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _i64, _f32, _f32, _f32, _f32, _f32, _vp]),
    "bz_mlp_batch": (ctypes.c_int, [_i32, _i32, ctypes.c_uint64, ctypes.c_uint64, _vp, _vp]),
    "bz_mlp_train_workspace": (_sz, [_i32]),
    "bz_mlp_train_step": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i32, _i32, ctypes.c_uint64,
                                         _i64, _f32, _f32, _f32, _f32, _f32, _vp, _vp, _sz, _vp]),
    "bz_seg_sample_energy_f32": (ctypes.c_int, [_P, Segments, _i32, _i32, _f64, _f64, _vp, _vp, ctypes.c_uint64, _vp]),
    "bz_seg_sample_energy_f64": (ctypes.c_int, [_P, Segments, _i32, _i32, _f64, _f64, _vp, _vp, ctypes.c_uint64, _vp]),
}


def exported_symbols():
    return sorted(_PROTOS)


def load():
    """Load libbz.so (once). Raises BzLibraryError if it is missing or broken."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise BzLibraryError(f"{LIB_PATH} is missing; build it with `python -m boltzmann_gb300.build` "
                             "(there is no CPU fallback)")
    try:
        lib = ctypes.CDLL(LIB_PATH)
    except OSError as e:
        raise BzLibraryError(f"cannot load {LIB_PATH}: {e}") from e
    for name, (res, args) in _PROTOS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def call(name, *args):
    """Call an entry point and raise BzError on a non-zero status."""
    rc = getattr(load(), name)(*args)
    if rc != BZ_OK:
        raise BzError(name, rc)
    return rc
