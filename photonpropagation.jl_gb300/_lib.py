"""ctypes binding of the C ABI declared in include/pp_gb300.h.

The shared library ``_lib/libpp_gb300.so`` is built in-tree by
``_build.build()``.  There is no CPU fallback: if the library is missing or no
CUDA device is present, calls fail loudly with :class:`PPError`.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import (POINTER, Structure, c_char_p, c_double, c_float, c_int32, c_int64,
                    c_uint32, c_uint64, c_void_p)

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG_DIR, "_lib", "libpp_gb300.so")

PP_OK = 0
PP_ERR_OVERFLOW = 1
PP_ERR_INVALID = -1
PP_ERR_CUDA = -2
PP_ERR_TIMEOUT = -3
PP_ERR_NOT_READY = -4
PP_ERR_NO_DEVICE = -5

PP_FLAG_OVERFLOW = 1
PP_FLAG_TIMEOUT = 2

# emitter kinds
PP_SRC_POINTLIKE_ISOTROPIC = 0
PP_SRC_EXTENDED_CHERENKOV = 1
PP_SRC_EXTENDED_CHERENKOV_NOSMEAR = 2
PP_SRC_POINTLIKE_CHERENKOV = 3
PP_SRC_CHERENKOV_TRACK = 4
PP_SRC_POINTLIKE_TIME_RANGE = 5
PP_SRC_COLLIMATED_ISOTROPIC = 6
PP_SRC_PENCIL = 7
PP_SRC_AXICONE = 8


class pp_source(Structure):
    _fields_ = [
        ("kind", c_int32), ("smear_table", c_int32), ("photons", c_int64),
        ("position", c_float * 3), ("time", c_float),
        ("direction", c_float * 3), ("time_end", c_float),
        ("long_a", c_float), ("long_b", c_float), ("long_lrad", c_float), ("length", c_float),
        ("angle", c_float), ("beam_divergence", c_float), ("cut_angle_cos", c_float),
        ("reserved1", c_float), ("first_photon", c_int64), ("reserved2", c_int64),
    ]


class pp_sphere(Structure):
    _fields_ = [("position", c_float * 3), ("radius", c_float)]


PP_PHASE_HG_ES = 0
PP_PHASE_HG_SL = 1


class pp_medium(Structure):
    _fields_ = [
        ("wl_min", c_float), ("wl_step", c_float), ("n_knots", c_int32), ("phase_kind", c_int32),
        ("scattering_length", POINTER(c_float)), ("group_velocity", POINTER(c_float)),
        ("absorption_length", POINTER(c_float)), ("phase_refractive_index", POINTER(c_float)),
        ("hg_g", c_float), ("es_b", c_float), ("hg_weight", c_float), ("reserved1", c_float),
    ]


class pp_tuning(Structure):
    _fields_ = [
        ("block_threads", c_int32), ("photons_per_thread", c_int32), ("ctas_per_sm", c_int32),
        ("precise_math", c_int32), ("cell_size", c_float), ("grid_in_global", c_int32),
        ("safety_cell", c_float), ("target_loop", c_int32),
    ]


PP_TARGET_SPHERE = 0
PP_TARGET_RECTANGLE = 1
PP_TARGET_DISC = 2
PP_TARGET_LINE = 3


class pp_target(Structure):
    _fields_ = [("position", c_float * 3), ("radius", c_float), ("length_x", c_float),
                ("length_y", c_float), ("kind", c_int32), ("reserved", c_int32)]


PP_PMT_HOMOGENEOUS = 0
PP_PMT_POM = 1
PP_PMT_DOM = 2
PP_PMT_MULTIPMT = 3
PP_POM_MAX_KNOTS = 128
PP_DOM_MAX_POLY = 16
PP_MULTIPMT_MAX_PMTS = 32


class pp_pmt_target(Structure):
    _fields_ = [("position", c_float * 3), ("radius", c_float), ("kind", c_int32),
                ("active_area", c_float)]


class pp_pom_model(Structure):
    _fields_ = [
        ("n_acc", c_int32), ("n_qe", c_int32),
        ("acc_wavelength", c_float * PP_POM_MAX_KNOTS), ("acc_group1", c_float * PP_POM_MAX_KNOTS),
        ("acc_group2", c_float * PP_POM_MAX_KNOTS), ("sigma_group1", c_float),
        ("sigma_group2", c_float), ("qe_wavelength", c_float * PP_POM_MAX_KNOTS),
        ("qe", c_float * PP_POM_MAX_KNOTS), ("pmt_dir", (c_float * 3) * 16),
        ("pmt_group", c_int32 * 16),
    ]


class pp_dom_model(Structure):
    _fields_ = [
        ("n_poly", c_int32), ("n_wl", c_int32), ("poly", c_float * PP_DOM_MAX_POLY),
        ("polymax", c_float), ("zenith_axis", c_float * 3), ("apply_wl_acceptance", c_int32),
        ("wl", c_float * PP_POM_MAX_KNOTS), ("wl_acc", c_float * PP_POM_MAX_KNOTS),
    ]


class pp_multipmt_model(Structure):
    _fields_ = [
        ("n_pmt", c_int32), ("n_qe", c_int32), ("pmt_area", c_float),
        ("pmt_dir_module", (c_float * 3) * PP_MULTIPMT_MAX_PMTS),
        ("pmt_dir", (c_float * 3) * PP_MULTIPMT_MAX_PMTS),
        ("qe_wavelength", c_float * PP_POM_MAX_KNOTS), ("qe", c_float * PP_POM_MAX_KNOTS),
    ]


class pp_detection_models(Structure):
    _fields_ = [("pom", POINTER(pp_pom_model)), ("dom", POINTER(pp_dom_model)),
                ("multipmt", POINTER(pp_multipmt_model))]


class pp_hit_record(Structure):
    _fields_ = [
        ("position", c_float * 3), ("wavelength", c_float),
        ("direction", c_float * 3), ("module_index", c_int32),
        ("dist_travelled", c_float), ("initial_direction", c_float * 3),
        ("abs_weight", c_float), ("n_steps", c_int32), ("source_index", c_int32),
        ("reserved", c_int32),
        ("time", c_double), ("photon_index", c_int64),
    ]


class pp_counters(Structure):
    _fields_ = [
        ("n_hits", c_uint64), ("n_ph_sim", c_uint64), ("photon_steps", c_uint64),
        ("work_next", c_uint64), ("err_flags", c_uint32), ("reserved", c_uint32 * 3),
    ]


class pp_hits(Structure):
    _fields_ = [
        ("position", c_void_p), ("direction", c_void_p), ("initial_direction", c_void_p),
        ("wavelength", c_void_p), ("time", c_void_p), ("dist_travelled", c_void_p),
        ("abs_weight", c_void_p), ("module_index", c_void_p), ("n_steps", c_void_p),
        ("source_index", c_void_p), ("photon_index", c_void_p),
    ]


assert ctypes.sizeof(pp_source) == 96
assert ctypes.sizeof(pp_hit_record) == 80
assert ctypes.sizeof(pp_counters) == 48

# Hit-record layout as a numpy structured dtype (for device buffers viewed on the host).
HIT_RECORD_DTYPE = [
    ("position", "<f4", (3,)), ("wavelength", "<f4"),
    ("direction", "<f4", (3,)), ("module_index", "<i4"),
    ("dist_travelled", "<f4"), ("initial_direction", "<f4", (3,)),
    ("abs_weight", "<f4"), ("n_steps", "<i4"), ("source_index", "<i4"), ("reserved", "<i4"),
    ("time", "<f8"), ("photon_index", "<i8"),
]


class PPError(RuntimeError):
    """A pp_* call failed; ``code`` is the pp_status value."""

    def __init__(self, code: int, message: str):
        super().__init__(f"[{code}] {message}")
        self.code = code


# name -> (restype, argtypes)
SIGNATURES = {
    "pp_version": (c_int32, []),
    "pp_last_error": (c_int32, [c_char_p, c_int32]),
    "pp_create": (c_int32, [POINTER(c_void_p), c_int32]),
    "pp_destroy": (c_int32, [c_void_p]),
    "pp_set_medium": (c_int32, [c_void_p, POINTER(pp_medium)]),
    "pp_set_spectrum": (c_int32, [c_void_p, POINTER(c_float), c_int32]),
    "pp_set_monochromatic": (c_int32, [c_void_p, c_float]),
    "pp_set_track_smear": (c_int32, [c_void_p, POINTER(c_float), c_int32]),
    "pp_set_track_smear_tables": (c_int32, [c_void_p, POINTER(c_float), c_int32, c_int32]),
    "pp_set_targets": (c_int32, [c_void_p, POINTER(pp_sphere), c_int32, c_float]),
    "pp_set_sources": (c_int32, [c_void_p, POINTER(pp_source), c_int32, c_float]),
    "pp_set_tuning": (c_int32, [c_void_p, POINTER(pp_tuning)]),
    "pp_get_tuning": (c_int32, [c_void_p, POINTER(pp_tuning)]),
    "pp_total_photons": (c_int32, [c_void_p, POINTER(c_int64)]),
    "pp_launch": (c_int32, [c_void_p, c_int64, c_int32, c_void_p, c_int64, c_void_p, c_void_p]),
    "pp_launch_graph": (c_int32, [c_void_p, c_int64, c_int32, c_void_p, c_int64, c_void_p,
                                  c_void_p]),
    "pp_launch_histogram": (c_int32, [c_void_p, c_int64, c_int32, c_void_p, c_void_p, c_int32,
                                      c_float, c_float, c_float, c_void_p, c_void_p]),
    "pp_propagate": (c_int32, [c_void_p, POINTER(pp_source), c_int32, c_int64, c_int32, c_float,
                               POINTER(pp_hits), c_int64, POINTER(c_int64), POINTER(c_int64)]),
    "pp_fetch_hits": (c_int32, [c_void_p, POINTER(pp_hits), c_int64]),
    "pp_device_memory": (c_int32, [c_int32, POINTER(c_int64), POINTER(c_int64)]),
    "pp_propagate_static": (c_int32, [POINTER(pp_medium), POINTER(c_float), c_int32, c_float,
                                      POINTER(c_float), c_int32, POINTER(pp_sphere), c_int32,
                                      c_float, POINTER(pp_source), c_int32, c_int64, c_int32,
                                      c_float, c_void_p, c_int64, POINTER(pp_counters),
                                      c_void_p]),
    "pp_hits_to_columns": (c_int32, [c_void_p, c_int64, POINTER(pp_hits), c_void_p]),
    "pp_mlp_create": (c_int32, [POINTER(c_void_p), c_int32, c_int32, c_int32, c_int32, c_int32,
                                c_int32, c_uint64]),
    "pp_mlp_destroy": (c_int32, [c_void_p]),
    "pp_mlp_num_params": (c_int32, [c_void_p, POINTER(c_int64)]),
    "pp_mlp_layout": (c_int32, [c_void_p, c_int32, POINTER(c_int64), POINTER(c_int64),
                                POINTER(c_int32), POINTER(c_int32)]),
    "pp_mlp_get_params": (c_int32, [c_void_p, POINTER(c_float), c_int64]),
    "pp_mlp_set_params": (c_int32, [c_void_p, POINTER(c_float), c_int64]),
    "pp_mlp_forward": (c_int32, [c_void_p, c_void_p, c_int32, c_void_p, c_void_p]),
    "pp_mlp_loss_grad": (c_int32, [c_void_p, c_void_p, c_void_p, c_void_p, c_int32,
                                   POINTER(c_float), POINTER(c_float), c_void_p]),
    "pp_mlp_train_steps": (c_int32, [c_void_p, c_void_p, c_void_p, c_void_p, c_int64, c_int32,
                                     c_int32, c_int64, c_int64, c_float, c_float, c_uint64,
                                     c_void_p]),
    "pp_mlp_step_count": (c_int32, [c_void_p, POINTER(c_int64)]),
    "pp_mlp_train_step": (c_int32, [c_void_p, c_void_p, c_void_p, c_void_p, c_int32, c_float,
                                    c_void_p]),
    "pp_mlp_last_loss": (c_int32, [c_void_p, POINTER(c_float)]),
    "pp_mlp_infer": (c_int32, [c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_void_p]),
    "pp_mlp_debug_infer_timeout": (c_int32, [c_void_p, c_void_p, c_int64, c_void_p, c_int64,
                                             c_void_p]),
    "pp_mlp_check": (c_int32, [c_void_p, c_void_p]),
    "pp_mlp_get_adam": (c_int32, [c_void_p, POINTER(c_float), POINTER(c_float), c_int64,
                                  POINTER(c_int64)]),
    "pp_mlp_set_adam": (c_int32, [c_void_p, POINTER(c_float), POINTER(c_float), c_int64,
                                  c_int64]),
    "pp_mlp_gemm_test": (c_int32, [c_void_p, c_int64, c_int32, c_void_p, c_int64, c_int32,
                                   c_int32, c_int32, c_int32, c_int32, c_void_p, c_int64,
                                   c_void_p]),
    "pp_autotune": (c_int32, [c_void_p, c_int64, c_int32, c_int64, POINTER(pp_tuning),
                              POINTER(c_double)]),
    "pp_make_hits_from_photons": (c_int32, [c_void_p, c_int64, POINTER(pp_pmt_target), c_int32,
                                            c_void_p, c_int64, c_void_p, c_void_p, c_void_p]),
    "pp_make_hits_from_photons_models": (c_int32, [c_void_p, c_int64, POINTER(pp_pmt_target),
                                                   c_int32, POINTER(pp_detection_models), c_int64,
                                                   c_void_p, c_void_p, c_void_p]),
    "pp_set_shaped_targets": (c_int32, [c_void_p, POINTER(pp_target), c_int32]),
    "pp_time_residuals": (c_int32, [c_void_p, c_int64, POINTER(c_double), c_int32, c_double,
                                    c_void_p, c_void_p]),
    "pp_debug_philox": (c_int32, [POINTER(c_uint32), c_int32, c_uint32, c_uint32,
                                  POINTER(c_uint32)]),
    "pp_debug_staging_timeout": (c_int32, [c_void_p, c_int64]),
    "pp_measure_fp32_peak": (c_int32, [c_int32, POINTER(c_double)]),
    "pp_grid_info": (c_int32, [c_void_p, POINTER(c_int32), POINTER(c_float), POINTER(c_float),
                               POINTER(c_int64), POINTER(c_int64)]),
}

_LIB = None


def lib_path() -> str:
    return LIB_PATH


def load(path: str | None = None):
    """Load the CUDA library (once).  Raises if it has not been built."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise ImportError(
            f"CUDA library not built: {p} is missing (run __graft_entry__.build() or "
            "python -m photonpropagation build); there is no CPU fallback")
    lib = ctypes.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _LIB = lib
    return lib


def last_error() -> str:
    lib = load()
    buf = ctypes.create_string_buffer(2048)
    lib.pp_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(rc: int, what: str = "") -> int:
    """Raise PPError for a negative status; return the status otherwise."""
    if rc < 0:
        raise PPError(rc, f"{what}: {last_error()}" if what else last_error())
    return rc
