"""ctypes binding of libfigpu.so (the C ABI of include/fi_gpu.h).

Loading fails loudly when the library is missing or no CUDA device is
usable: there is no CPU path.
"""
import ctypes as C
import os

from . import build as _build

FI_OK, FI_E_NAN, FI_E_LARGE, FI_E_STEP, FI_E_OOM, FI_E_CONFIG, FI_E_CUDA, FI_E_TIMEOUT, FI_E_ARG, FI_E_STATE, \
    FI_E_SIZE, FI_E_CANCELLED = range(12)
FI_STATIC_MAX_N = 256
FI_PREC_FP64, FI_PREC_MIXED = 0, 1

ERRORS = {1: "FI_E_NAN", 2: "FI_E_LARGE", 3: "FI_E_STEP", 4: "FI_E_OOM", 5: "FI_E_CONFIG", 6: "FI_E_CUDA",
          7: "FI_E_TIMEOUT", 8: "FI_E_ARG", 9: "FI_E_STATE", 10: "FI_E_SIZE", 11: "FI_E_CANCELLED"}

FIELDS = {
    "z_bed": 0, "dwdt": 1, "w": 2, "we": 3, "Haf": 4, "Hice": 5, "z_ss": 6, "dz_ss": 7,
    "canom_load": 8, "canom_full": 9, "mass_anom": 10, "maskocean": 11, "maskgrounded": 12,
    "maskcontinent": 13, "canom_mantle": 14, "canom_litho": 15, "canom_seawater": 16,
    "canom_ice": 17, "x": 18, "kappa": 19, "D_lith": 20, "eta_eff": 21, "R": 22,
    "maskactive": 23, "GE": 24, "GN": 25,
}

EXPORTS = ["fi_create", "fi_destroy", "fi_dims", "fi_set_fields", "fi_set_kernels", "fi_init_ref",
           "fi_init_state", "fi_update", "fi_update_async", "fi_synchronize", "fi_bsl_update",
           "fi_get_field", "fi_get_scalars", "fi_lvelva", "fi_convolve", "fi_state_size",
           "fi_state_export", "fi_state_import", "fi_last_error", "fi_version", "fi_stream",
           "fi_launch_count", "fi_profile", "fi_profile_read", "fi_engine_trace", "fi_lvelva_static",
           "fi_padded_dims", "fi_serve_create", "fi_serve_submit", "fi_serve_info", "fi_serve_wait",
           "fi_serve_result", "fi_serve_clock", "fi_serve_destroy", "fi_batch_update", "fi_batch_synchronize",
           "fi_batch_create", "fi_batch_step", "fi_batch_wait", "fi_batch_destroy", "fi_elva_disk",
           "fi_batch_set_priority", "fi_set_rheology", "fi_output_bytes", "fi_output_async",
           "fi_output_wait", "fi_batch_autotune", "fi_set_stream", "fi_set_max_rejections", "fi_serve_cancel",
           "fi_metrics_json"]

PROFILE_KERNELS = ["flexure", "rows_fwd", "cols_hartley", "rows_inv", "conv_rows_fwd", "conv_cols",
                   "conv_rows_inv", "rk_stage", "rk_final", "upd_begin", "upd_masks", "upd_litho",
                   "upd_load", "upd_end", "control", "ts", "engine"]


class FiParams(C.Structure):
    _fields_ = [
        ("method", C.c_int32), ("interactive_sealevel", C.c_int32), ("include_elastic", C.c_int32),
        ("heterogeneous_ssh", C.c_int32), ("correct_compression", C.c_int32),
        ("lithosphere", C.c_int32), ("mantle", C.c_int32), ("layering", C.c_int32),
        ("lumping", C.c_int32), ("visc_scaling_method", C.c_int32), ("nl", C.c_int32),
        ("dt_method", C.c_int32), ("stage_mode", C.c_int32), ("nx_target", C.c_int32),
        ("ny_target", C.c_int32), ("precision", C.c_int32),
        ("dt_diagnostics", C.c_double), ("min_pad", C.c_double), ("viscosity_scaling", C.c_double),
        ("zl", C.c_double * 8), ("viscosities", C.c_double * 8), ("dl", C.c_double),
        ("eta_ref", C.c_double), ("E", C.c_double), ("nu", C.c_double), ("rho_water", C.c_double),
        ("rho_ice", C.c_double), ("rho_seawater", C.c_double), ("rho_uppermantle", C.c_double),
        ("rho_litho", C.c_double), ("g", C.c_double), ("r_earth", C.c_double),
        ("m_earth", C.c_double), ("atol", C.c_double), ("rtol", C.c_double),
        ("dt_min", C.c_double), ("dt_max", C.c_double), ("dt_init", C.c_double), ("q", C.c_double), ("tau", C.c_double),
    ]


class FiRheology(C.Structure):
    """fi_rheology: the arrays of a rheology file (x fastest)."""
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
                ("xc", C.POINTER(C.c_double)), ("yc", C.POINTER(C.c_double)), ("zc", C.POINTER(C.c_double)),
                ("litho_thickness", C.POINTER(C.c_double)), ("litho_thickness_scaling", C.c_double),
                ("log10_viscosity", C.POINTER(C.c_double)), ("stddev_log10_viscosity", C.POINTER(C.c_double)),
                ("stddev_scaling", C.c_int32), ("rheo_smoothing_radius", C.c_double)]


class FiBsl(C.Structure):
    _fields_ = [
        ("method", C.c_int32), ("constant_ocean_surface", C.c_int32), ("n_series", C.c_int32),
        ("n_aocean", C.c_int32), ("bsl_init", C.c_double), ("bsl_now", C.c_double),
        ("A_ocean_now", C.c_double), ("A_ocean_pd", C.c_double), ("time", C.c_double),
        ("series_t", C.POINTER(C.c_double)), ("series_v", C.POINTER(C.c_double)),
        ("bsl_vec", C.POINTER(C.c_double)), ("aocean_vec", C.POINTER(C.c_double)),
    ]


_dp = C.POINTER(C.c_double)
_u8 = C.POINTER(C.c_uint8)


class FiOut(C.Structure):
    _fields_ = [(k, _dp) for k in ("z_bed", "z_ss", "dz_ss", "w", "we", "dwdt", "canom_full", "Hice")] + \
               [(k, _u8) for k in ("maskocean", "maskgrounded", "maskcontinent")]


class FiRequest(C.Structure):
    _fields_ = [("p", FiParams), ("nx_ice", C.c_int32), ("ny_ice", C.c_int32), ("dx", C.c_double),
                ("dy", C.c_double), ("z_bed", _dp), ("H_ref", _dp), ("H_ice", _dp), ("D_lith", _dp), ("eta_eff", _dp),
                ("R", _dp), ("maskactive", _u8), ("t0", C.c_double), ("t_end", C.c_double),
                ("dtt", C.c_double), ("bsl", C.c_double)]


class FiRequestInfo(C.Structure):
    _fields_ = [("state", C.c_int32), ("status", C.c_int32), ("updates", C.c_int64), ("t_submit", C.c_double),
                ("t_admit", C.c_double), ("t_done", C.c_double), ("error", C.c_char * 128)]


_LIB = None


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load libfigpu.so (building it in-tree if needed)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.LIB
    if build_if_missing and not _build.up_to_date():
        path = _build.build()
    if not os.path.exists(path):
        raise RuntimeError("libfigpu.so is not built (run __graft_entry__.build())")
    L = C.CDLL(path)
    H = C.c_void_p
    L.fi_create.argtypes = [C.POINTER(FiParams), C.c_int, C.c_int, C.c_double, C.c_double, _dp, C.POINTER(H)]
    L.fi_destroy.argtypes = [H]
    L.fi_dims.argtypes = [H, C.POINTER(C.c_int32)]
    L.fi_set_fields.argtypes = [H, _dp, _dp, _dp, _u8]
    L.fi_set_rheology.argtypes = [H, C.POINTER(FiRheology)]
    L.fi_output_bytes.argtypes = [H]
    L.fi_output_bytes.restype = C.c_int64
    L.fi_output_async.argtypes = [H, C.c_void_p]
    L.fi_output_wait.argtypes = [H]
    L.fi_set_kernels.argtypes = [H, _dp, _dp]
    L.fi_init_ref.argtypes = [H, _dp, _dp, C.c_double, _dp]
    L.fi_init_state.argtypes = [H, _dp, _dp, C.c_double, C.POINTER(FiBsl)]
    L.fi_update.argtypes = [H, _dp, C.c_double, C.POINTER(FiBsl), C.POINTER(FiOut)]
    L.fi_update_async.argtypes = [H, C.c_void_p, C.c_double, C.POINTER(FiBsl)]
    L.fi_synchronize.argtypes = [H]
    L.fi_set_max_rejections.argtypes = [H, C.c_int64]
    L.fi_metrics_json.argtypes = [H, C.c_char_p, C.c_size_t]
    L.fi_bsl_update.argtypes = [C.POINTER(FiBsl), C.c_double]
    L.fi_get_field.argtypes = [H, C.c_int, _dp]
    L.fi_get_scalars.argtypes = [H, _dp]
    L.fi_lvelva.argtypes = [H, _dp, _dp, _dp]
    L.fi_convolve.argtypes = [H, C.c_int, _dp, _dp]
    _v = C.c_void_p
    L.fi_lvelva_static.argtypes = [_v, _v, _v, _v, _v, _v, _v, _v, _v, C.c_int, C.c_int, C.c_double,
                                   C.c_double, C.c_double, C.c_double, C.c_double, _v, _v]
    L.fi_state_size.argtypes = [H]
    L.fi_state_size.restype = C.c_size_t
    L.fi_state_export.argtypes = [H, _dp]
    L.fi_state_import.argtypes = [H, _dp]
    L.fi_stream.argtypes = [H]
    L.fi_stream.restype = C.c_void_p
    L.fi_launch_count.argtypes = [H]
    L.fi_launch_count.restype = C.c_longlong
    L.fi_engine_trace.argtypes = [H, C.c_void_p, C.c_int]
    L.fi_profile.argtypes = [H, C.c_int]
    L.fi_profile_read.argtypes = [H, _dp, C.POINTER(C.c_longlong), C.c_int]
    L.fi_padded_dims.argtypes = [C.POINTER(FiParams), C.c_int, C.c_int, C.c_double, C.c_double,
                                 C.POINTER(C.c_int32)]
    L.fi_serve_create.argtypes = [C.c_int, C.c_double, C.POINTER(H)]
    L.fi_serve_submit.argtypes = [H, C.POINTER(FiRequest), C.POINTER(C.c_uint64)]
    L.fi_serve_info.argtypes = [H, C.c_uint64, C.POINTER(FiRequestInfo)]
    L.fi_serve_wait.argtypes = [H, C.c_uint64, C.c_double, C.POINTER(FiRequestInfo)]
    L.fi_serve_result.argtypes = [H, C.c_uint64, _dp, _dp]
    L.fi_serve_clock.argtypes = [H]
    L.fi_serve_clock.restype = C.c_double
    L.fi_serve_destroy.argtypes = [H]
    L.fi_serve_cancel.argtypes = [H, C.c_uint64]
    L.fi_batch_update.argtypes = [C.POINTER(H), C.c_int, C.c_double, C.POINTER(FiBsl)]
    L.fi_batch_synchronize.argtypes = [C.POINTER(H), C.c_int, C.POINTER(C.c_int32)]
    L.fi_batch_create.argtypes = [C.POINTER(H), C.c_int, C.POINTER(H)]
    L.fi_batch_step.argtypes = [H, C.c_double, C.POINTER(FiBsl)]
    L.fi_batch_set_priority.argtypes = [H, C.c_int]
    L.fi_batch_autotune.argtypes = [H, C.POINTER(C.c_int32)]
    L.fi_set_stream.argtypes = [H, C.c_void_p]
    L.fi_batch_wait.argtypes = [H, C.POINTER(C.c_int32)]
    L.fi_batch_destroy.argtypes = [H]
    L.fi_elva_disk.argtypes = [C.c_int, C.c_int] + [C.c_double] * 9 + [_dp]
    L.fi_last_error.argtypes = [H]
    L.fi_last_error.restype = C.c_char_p
    _LIB = L
    return L


class FiError(RuntimeError):
    def __init__(self, code, msg=""):
        super().__init__("%s (%d): %s" % (ERRORS.get(code, "?"), code, msg))
        self.code = code
