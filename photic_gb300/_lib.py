"""ctypes binding of libphotic_gb300.so (the C ABI in include/photic.h and
include/photic_nc.h).

The structs below mirror include/photic.h field for field.  Loading fails
loudly when the library has not been built: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libphotic_gb300.so")

MAX_BANDS = 8
MAX_SCENES = 8
MAX_HSTARTS = 32

OK, ERR_INVALID, ERR_CUDA, ERR_NOMEM, ERR_TIMEOUT, ERR_UNSUPPORTED, ERR_IO = range(7)
PREC_FP64, PREC_DF64, PREC_FP32, PREC_GUARDED = 0, 1, 2, 3
LAYOUT_REFERENCE, LAYOUT_SCENE_B = 0, 1
TUNE_INVERT, TUNE_JOINT = 0, 1
PX_FITTED, PX_MASKED, PX_INVALID = 0, 1, 2
PX_CONVERGED = 0x100
PX_SERVED = 0x200
PX_HOT = 0x400


class photic_config(C.Structure):
    _fields_ = [
        ("n_bands", C.c_int32),
        ("wavelengths", C.c_double * MAX_BANDS),
        ("theta_sun_deg", C.c_double),
        ("theta_view_deg", C.c_double),
        ("h_tide", C.c_double),
        ("nodata_value", C.c_float),
        ("reqmin", C.c_double),
        ("konvge", C.c_int32),
        ("kcount", C.c_int32),
        ("n_hstarts", C.c_int32),
        ("hstarts", C.c_double * MAX_HSTARTS),
        ("early_exit_per_scene", C.c_double),
        ("precision", C.c_int32),
        ("layout", C.c_int32),
        ("block_threads", C.c_int32),
        ("blocks_per_sm", C.c_int32),
        ("seed_step_scale", C.c_double),
    ]


class photic_outputs(C.Structure):
    _fields_ = [
        ("depth", C.c_void_p),
        ("depth_f64", C.c_void_p),
        ("P", C.c_void_p),
        ("G", C.c_void_p),
        ("X", C.c_void_p),
        ("bottom_albedo", C.c_void_p),
        ("model_error", C.c_void_p),
        ("rrs_error", C.c_void_p),
        ("K_min", C.c_void_p),
        ("iod", C.c_void_p),
        ("evals", C.c_void_p),
        ("evals_kept", C.c_void_p),
        ("status", C.c_void_p),
        ("params", C.c_void_p),
        ("bottom_percent", C.c_void_p),
        ("bottom_type", C.c_void_p),
    ]


class photic_lut_config(C.Structure):
    _fields_ = [
        ("n_lut", C.c_int32),
        ("n_chains", C.c_int64),
        ("use_noise", C.c_int32),
        ("rrs_noise", C.c_double * MAX_BANDS),
    ]


class photic_nc_grid_info(C.Structure):
    """include/photic_nc.h"""
    _fields_ = [
        ("ncols", C.c_int32),
        ("nrows", C.c_int32),
        ("add_offset", C.c_float),
        ("scale_factor", C.c_float),
        ("missing_value", C.c_int16),
        ("has_missing_value", C.c_int32),
        ("spval", C.c_double),
        ("has_spval", C.c_int32),
        ("format", C.c_int32),
    ]


class PhoticError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"photic error {code}: {msg}")
        self.code = code


_lib = None

# name -> (restype, argtypes)
_SIGS = {
    "photic_version": (C.c_char_p, []),
    "photic_last_error": (C.c_char_p, []),
    "photic_config_default": (None, [C.POINTER(photic_config)]),
    "photic_config_check": (C.c_int, [C.POINTER(photic_config)]),
    "photic_invert_batch": (C.c_int, [C.POINTER(photic_config), C.c_void_p, C.c_int64,
                                      C.c_int64, C.c_int64, C.c_void_p,
                                      C.POINTER(photic_outputs), C.c_void_p]),
    "photic_invert_batch_ordered": (C.c_int, [C.POINTER(photic_config), C.c_void_p, C.c_int64,
                                              C.c_int64, C.c_int64, C.c_void_p, C.c_void_p,
                                              C.POINTER(photic_outputs), C.c_void_p]),
    "photic_invert_batch_noalloc": (C.c_int, [C.POINTER(photic_config), C.c_void_p, C.c_int64,
                                              C.c_int64, C.c_int64, C.c_void_p,
                                              C.POINTER(photic_outputs), C.c_void_p]),
    "photic_joint_invert_batch": (C.c_int, [C.POINTER(photic_config), C.c_void_p, C.c_void_p,
                                            C.c_void_p, C.c_int64, C.c_int64,
                                            C.POINTER(photic_outputs), C.c_void_p]),
    "photic_cost_batch": (C.c_int, [C.POINTER(photic_config), C.c_void_p, C.c_void_p,
                                    C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]),
    "photic_generate_scene": (C.c_int, [C.POINTER(photic_config), C.c_uint64, C.c_int64,
                                        C.c_int64, C.c_double, C.c_double, C.c_void_p,
                                        C.c_void_p, C.c_void_p]),
    "photic_generate_field": (C.c_int, [C.POINTER(photic_config), C.c_uint64, C.c_int64,
                                        C.c_int64, C.c_int64, C.c_int64, C.c_double, C.c_double,
                                        C.c_void_p, C.c_void_p, C.c_void_p]),
    "photic_joint_counts": (C.c_int, [C.c_uint64, C.c_int64, C.c_int32, C.c_int32, C.c_void_p,
                                      C.c_void_p]),
    "photic_generate_joint": (C.c_int, [C.POINTER(photic_config), C.c_uint64, C.c_int64,
                                        C.c_void_p, C.c_double, C.c_double, C.c_double,
                                        C.c_double, C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_void_p]),
    "photic_interp_1d": (C.c_double, [C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int32,
                                      C.c_double]),
    "photic_band_constants": (C.c_int, [C.POINTER(photic_config), C.POINTER(C.c_double)]),
    "photic_sync": (C.c_int, [C.c_void_p]),
    "photic_forward_batch": (C.c_int, [C.POINTER(photic_config), C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p,
                                       C.c_void_p]),
    "photic_measure_peaks": (C.c_int, [C.POINTER(C.c_double)] * 3),
    "photic_region_invert_batch": (C.c_int, [C.POINTER(photic_config), C.c_void_p, C.c_int32,
                                             C.c_int32, C.c_int32, C.POINTER(photic_outputs),
                                             C.c_void_p]),
    "photic_bottom_reflectances": (C.c_int, [C.POINTER(photic_config), C.c_int32,
                                             C.POINTER(C.c_double)]),
    "photic_region_fit_batch": (C.c_int, [C.POINTER(photic_config), C.c_void_p, C.c_int32,
                                          C.POINTER(C.c_double), C.c_int32, C.c_int32,
                                          C.c_int32, C.c_int32, C.c_void_p,
                                          C.POINTER(photic_outputs), C.c_void_p]),
    "photic_lut_config_default": (None, [C.POINTER(photic_lut_config)]),
    "photic_lut_default_chains": (C.c_int64, [C.POINTER(photic_config)]),
    "photic_lut_invert_batch": (C.c_int, [C.POINTER(photic_config), C.POINTER(photic_lut_config),
                                          C.c_void_p, C.c_int64, C.c_void_p, C.c_float,
                                          C.POINTER(photic_outputs),
                                          C.c_void_p, C.c_void_p, C.c_void_p,
                                          C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                          C.c_void_p]),
    "photic_region_lut_invert_batch": (C.c_int, [C.POINTER(photic_config),
                                                 C.POINTER(photic_lut_config), C.c_void_p,
                                                 C.c_int32, C.POINTER(C.c_double), C.c_int32,
                                                 C.c_int32, C.c_int32, C.c_int32,
                                                 C.POINTER(C.c_double), C.c_void_p, C.c_float,
                                                 C.POINTER(photic_outputs), C.c_void_p,
                                                 C.c_void_p, C.c_void_p,
                                                 C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                                 C.c_void_p]),
    "photic_region_lut_default_chains": (C.c_int64, [C.POINTER(photic_config), C.c_int32,
                                                     C.c_int32, C.c_int32]),
    "photic_region_depth_sigma": (C.c_int, [C.POINTER(photic_config), C.c_void_p, C.c_int32,
                                            C.POINTER(C.c_double), C.c_int32, C.c_int32,
                                            C.c_int32, C.c_int32, C.c_void_p,
                                            C.POINTER(C.c_double), C.c_int32, C.c_uint64,
                                            C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                            C.c_void_p]),
    "photic_depth_sigma": (C.c_int, [C.POINTER(photic_config), C.c_void_p, C.c_int64, C.c_void_p,
                                     C.POINTER(C.c_double), C.c_int32, C.c_uint64, C.c_void_p,
                                     C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "photic_autotune": (C.c_int, [C.POINTER(photic_config), C.c_int32, C.c_int64,
                                  C.POINTER(C.c_double), C.c_int32, C.POINTER(C.c_int32)]),
    "photic_set_counter": (C.c_int, [C.c_void_p]),
    "photic_set_guard_stats": (C.c_int, [C.c_void_p]),
    "photic_surrogate_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_uint64]),
    "photic_surrogate_destroy": (C.c_int, [C.c_void_p]),
    "photic_surrogate_num_params": (C.c_int32, []),
    "photic_surrogate_params": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32]),
    "photic_surrogate_grads": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32,
                                         C.c_void_p, C.c_void_p, C.c_void_p]),
    "photic_surrogate_train_step": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32,
                                              C.c_float, C.c_void_p, C.c_void_p]),
    "photic_surrogate_infer": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p,
                                         C.c_void_p]),
    "photic_surrogate_seed": (C.c_int, [C.c_void_p, C.POINTER(photic_config), C.c_void_p,
                                        C.c_int64, C.c_double, C.c_void_p, C.c_void_p,
                                        C.c_void_p]),
    "photic_surrogate_seed_polished": (C.c_int, [C.c_void_p, C.POINTER(photic_config),
                                                 C.c_void_p, C.c_int64, C.c_double, C.c_int32,
                                                 C.c_void_p, C.c_void_p, C.c_void_p]),
    "photic_seed_polished_heuristic": (C.c_int, [C.POINTER(photic_config), C.c_void_p,
                                                 C.c_int64, C.c_double, C.c_double, C.c_int32,
                                                 C.c_void_p, C.c_void_p, C.c_void_p]),
    "photic_nc_read_info": (C.c_int, [C.c_char_p, C.POINTER(photic_nc_grid_info)]),
    "photic_nc_read_raw": (C.c_int, [C.c_char_p, C.POINTER(photic_nc_grid_info), C.c_void_p,
                                     C.c_void_p, C.c_void_p]),
    "photic_nc_write_raw": (C.c_int, [C.c_char_p, C.POINTER(photic_nc_grid_info), C.c_void_p,
                                      C.c_void_p, C.c_void_p]),
    "photic_nc_unpack_bands": (C.c_int, [C.POINTER(C.c_void_p), C.POINTER(photic_nc_grid_info),
                                         C.c_int32, C.c_int64, C.c_void_p, C.c_void_p]),
    "photic_nc_pack": (C.c_int, [C.c_void_p, C.c_int64, C.c_double, C.c_void_p,
                                 C.POINTER(photic_nc_grid_info), C.c_void_p]),
    "photic_nc_read_bands": (C.c_int, [C.POINTER(C.c_char_p), C.c_int32, C.c_void_p, C.c_int64,
                                       C.POINTER(photic_nc_grid_info), C.c_void_p, C.c_void_p,
                                       C.c_void_p]),
    "photic_nc_write_grid": (C.c_int, [C.c_char_p, C.c_void_p, C.c_int32, C.c_int32, C.c_void_p,
                                       C.c_void_p, C.c_double, C.c_void_p]),
    "read_nc": (None, [C.c_char_p, C.POINTER(C.POINTER(C.POINTER(C.c_float))),
                       C.POINTER(C.c_int), C.POINTER(C.c_int),
                       C.POINTER(C.POINTER(C.c_float)), C.POINTER(C.POINTER(C.c_float)),
                       C.POINTER(C.c_double)]),
    "write_nc": (None, [C.c_char_p, C.POINTER(C.POINTER(C.c_float)), C.c_int, C.c_int,
                        C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_double]),
    "photic_gemm_bf16": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_void_p,
                                   C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_void_p]),
    "photic_gemm_bf16_strides": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32,
                                           C.c_void_p, C.c_int32, C.c_int32, C.c_int32,
                                           C.c_int32, C.c_int32, C.c_int32, C.c_void_p]),
}


def lib() -> C.CDLL:
    """The loaded library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; "
                "g.build()'` (nvcc for sm_103a). There is no CPU fallback.")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def exported_symbols():
    return list(_SIGS)


def check(rc: int) -> None:
    if rc != OK:
        raise PhoticError(rc, lib().photic_last_error().decode(errors="replace"))
