"""ctypes binding of libimfcs_gb300.so (the in-tree CUDA library).

The library is the product; this module only declares its C ABI
(include/imfcs_gb300.h).  Loading fails loudly when the library is missing:
there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libimfcs_gb300.so")

NPARAM = 11
NCONST = 9

BLEACH_NONE, BLEACH_SINGLE_EXP, BLEACH_DOUBLE_EXP, BLEACH_POLYNOMIAL = 0, 1, 2, 3
MODEL_GAUSS_2D, MODEL_ACF_1D, MODEL_LINEAR_1D = 1, 2, 3

_lib = None

# Every symbol include/imfcs_gb300.h declares.
EXPORTS = [
    "imfcs_is_cuda_available", "imfcs_get_cuda_version", "imfcs_get_last_error", "imfcs_reset_gpu",
    "imfcs_is_binning_memory_sufficient", "imfcs_calc_binning", "imfcs_calc_data_bleach_correction",
    "imfcs_is_acf_memory_sufficient", "imfcs_calc_acf", "imfcs_fit", "imfcs_chanum",
    "imfcs_plan_create", "imfcs_plan_destroy", "imfcs_plan_scratch_bytes", "imfcs_plan_execute",
    "imfcs_plan_execute_host", "imfcs_diffusion_law", "imfcs_simulate", "imfcs_plan_bleach_params",
    "imfcs_plan_set_timing", "imfcs_plan_stage_times", "imfcs_plan_kernel_launches",
    "imfcs_fit_device_noalloc",
    "imfcs_surrogate_param_count", "imfcs_surrogate_create", "imfcs_surrogate_destroy",
    "imfcs_surrogate_get_params", "imfcs_surrogate_set_params", "imfcs_surrogate_features",
    "imfcs_surrogate_gradients", "imfcs_surrogate_train", "imfcs_surrogate_predict",
    "imfcs_plan_set_surrogate", "imfcs_plan_surrogate_stats", "imfcs_plan_set_background_image",
    "imfcs_plan_execute_host_async", "imfcs_plan_synchronize", "imfcs_psf_calibration",
    "imfcs_plan_set_corr_tile", "imfcs_plan_get_corr_tile", "imfcs_plan_autotune",
    "imfcs_batch_create", "imfcs_batch_destroy", "imfcs_batch_execute", "imfcs_batch_synchronize",
    "imfcs_batch_autotune", "imfcs_batch_job_info", "imfcs_batch_lanes", "imfcs_batch_scratch_bytes",
    "imfcs_batch_kernel_launches",
    "imfcs_tiff_open", "imfcs_tiff_read", "imfcs_tiff_read_device", "imfcs_tiff_close", "imfcs_background_stats",
    "imfcs_bands_create", "imfcs_bands_destroy", "imfcs_bands_geometry", "imfcs_bands_plan", "imfcs_bands_execute",
    "imfcs_band_window", "imfcs_measure_fp32_fma_rate", "imfcs_bands_set_background_image",
]


class ImfcsError(RuntimeError):
    pass


class ACFParameters(C.Structure):
    """imfcs_acf_parameters == GpufitImFCS.ACFParameters (GpufitImFCS.java:453-486)."""
    _fields_ = [
        ("width", C.c_int), ("height", C.c_int), ("win_star", C.c_int), ("hin_star", C.c_int),
        ("w_temp", C.c_int), ("h_temp", C.c_int), ("pixbinX", C.c_int), ("pixbinY", C.c_int),
        ("binningX", C.c_int), ("binningY", C.c_int), ("firstframe", C.c_int),
        ("lastframe", C.c_int), ("framediff", C.c_int), ("cfXDistance", C.c_int),
        ("cfYDistance", C.c_int), ("correlatorp", C.c_double), ("correlatorq", C.c_double),
        ("frametime", C.c_double), ("background", C.c_int), ("mtab1", C.c_double),
        ("mtabchanumminus1", C.c_double), ("sampchanumminus1", C.c_double), ("chanum", C.c_int),
        ("isNBcalculation", C.c_int), ("bleachcorr_gpu", C.c_int), ("bleachcorr_order", C.c_int),
        ("nopit", C.c_int), ("ave", C.c_int),
    ]


class Config(C.Structure):
    """imfcs_config."""
    _fields_ = [
        ("width", C.c_int), ("height", C.c_int), ("frames", C.c_int),
        ("first", C.c_int), ("num", C.c_int),
        ("out_w", C.c_int), ("out_h", C.c_int), ("map_x0", C.c_int), ("map_y0", C.c_int),
        ("binx", C.c_int), ("biny", C.c_int), ("pixbinx", C.c_int), ("pixbiny", C.c_int),
        ("cfx", C.c_int), ("cfy", C.c_int), ("background", C.c_int),
        ("p", C.c_int), ("q", C.c_int), ("frametime", C.c_double),
        ("bleach", C.c_int), ("poly_order", C.c_int),
        ("gls", C.c_int), ("bayes", C.c_int), ("do_fit", C.c_int),
        ("fitstart", C.c_int), ("fitend", C.c_int), ("max_iter", C.c_int),
        ("init", C.c_double * NPARAM), ("free_mask", C.c_int * NPARAM),
        ("cst", C.c_double * NCONST),
    ]


class CorrTile(C.Structure):
    """imfcs_corr_tile."""
    _fields_ = [("cta", C.c_int), ("seg_extra", C.c_int), ("tail_extra", C.c_int), ("ms", C.c_float)]


class Outputs(C.Structure):
    """imfcs_outputs (raw pointers, device or host depending on the call)."""
    _fields_ = [(n, C.c_void_p) for n in (
        "acf", "var", "sd", "blocked_ind", "blocked_ok", "nb_mean", "nb_cov", "fitres", "chi2",
        "fitted", "iterations", "bayes_prob", "covmats")]


class SimParams(C.Structure):
    """imfcs_sim_params."""
    _fields_ = [
        ("width", C.c_int), ("height", C.c_int), ("frames", C.c_int), ("frametime", C.c_double),
        ("steps_per_frame", C.c_int), ("pixel_size", C.c_double), ("psf_radius", C.c_double),
        ("density", C.c_double), ("d1", C.c_double), ("d2", C.c_double), ("fraction2", C.c_double),
        ("cps", C.c_double), ("tau_bleach", C.c_double), ("offset", C.c_int),
        ("read_noise", C.c_double), ("margin", C.c_double), ("seed", C.c_uint64),
    ]


def _declare(L: C.CDLL) -> None:
    vp, ip, dp = C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double)
    L.imfcs_is_cuda_available.restype = C.c_int
    L.imfcs_get_cuda_version.argtypes = [ip, ip]
    L.imfcs_get_last_error.restype = C.c_char_p
    L.imfcs_reset_gpu.restype = C.c_int
    L.imfcs_is_binning_memory_sufficient.argtypes = [C.POINTER(ACFParameters)]
    L.imfcs_calc_binning.argtypes = [vp, vp, C.POINTER(ACFParameters)]
    L.imfcs_calc_data_bleach_correction.argtypes = [vp, vp, C.POINTER(ACFParameters)]
    L.imfcs_is_acf_memory_sufficient.argtypes = [C.POINTER(ACFParameters)]
    L.imfcs_calc_acf.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp, vp, C.POINTER(ACFParameters)]
    L.imfcs_fit.argtypes = [C.c_int, C.c_int, vp, vp, C.c_int, vp, C.c_float, C.c_int, C.c_int, vp,
                            C.c_int, C.c_size_t, vp, vp, vp, vp, vp]
    L.imfcs_chanum.argtypes = [C.c_int, C.c_int]
    L.imfcs_plan_create.argtypes = [C.POINTER(Config), C.POINTER(C.c_void_p)]
    L.imfcs_plan_destroy.argtypes = [vp]
    L.imfcs_plan_scratch_bytes.restype = C.c_size_t
    L.imfcs_plan_scratch_bytes.argtypes = [vp]
    L.imfcs_plan_execute.argtypes = [vp, vp, C.POINTER(Outputs), vp]
    L.imfcs_plan_execute_host.argtypes = [vp, vp, C.POINTER(Outputs), vp]
    L.imfcs_diffusion_law.argtypes = [C.POINTER(Config), vp, C.c_int, C.c_int, C.c_int, C.c_double,
                                      C.c_double, dp, dp, vp]
    L.imfcs_simulate.argtypes = [C.POINTER(SimParams), vp, vp, vp]
    L.imfcs_plan_bleach_params.argtypes = [vp, vp, C.c_int]
    L.imfcs_plan_set_timing.argtypes = [vp, C.c_int]
    L.imfcs_plan_stage_times.argtypes = [vp, vp, C.c_int]
    L.imfcs_plan_kernel_launches.argtypes = [vp]
    L.imfcs_fit_device_noalloc.argtypes = [C.c_int, C.c_int, vp, vp, C.c_int, vp, C.c_float, C.c_int, C.c_int,
                                           vp, vp, vp, vp, vp, vp, vp]
    L.imfcs_surrogate_param_count.restype = C.c_size_t
    L.imfcs_surrogate_param_count.argtypes = []
    L.imfcs_surrogate_create.argtypes = [C.c_uint64, C.POINTER(C.c_void_p)]
    L.imfcs_surrogate_destroy.argtypes = [vp]
    L.imfcs_surrogate_get_params.argtypes = [vp, vp]
    L.imfcs_surrogate_set_params.argtypes = [vp, vp]
    L.imfcs_surrogate_features.argtypes = [C.c_int, C.c_int, vp, vp, vp, vp]
    L.imfcs_surrogate_gradients.argtypes = [vp, vp, vp, C.c_int, vp, dp]
    L.imfcs_surrogate_train.argtypes = [vp, vp, vp, C.c_int, C.c_int, C.c_int, C.c_float, C.c_uint64, vp, vp]
    L.imfcs_surrogate_predict.argtypes = [vp, vp, C.c_int, vp, vp]
    L.imfcs_plan_set_surrogate.argtypes = [vp, vp, C.c_int]
    L.imfcs_plan_surrogate_stats.argtypes = [vp, ip, ip]
    L.imfcs_plan_set_background_image.argtypes = [vp, vp]
    L.imfcs_plan_execute_host_async.argtypes = [vp, vp, C.POINTER(Outputs), vp]
    L.imfcs_plan_synchronize.argtypes = [vp, vp]
    L.imfcs_psf_calibration.argtypes = [C.POINTER(Config), vp, C.c_int, C.c_int, dp, C.c_int, C.c_double, dp, vp]
    L.imfcs_plan_set_corr_tile.argtypes = [vp, C.c_int, C.c_int, C.c_int]
    L.imfcs_plan_get_corr_tile.argtypes = [vp, ip, ip, ip]
    L.imfcs_plan_autotune.argtypes = [vp, vp, C.POINTER(Outputs), vp, C.POINTER(CorrTile), C.c_int, ip]
    L.imfcs_batch_create.argtypes = [C.POINTER(Config), C.c_int, C.c_int, C.POINTER(C.c_void_p)]
    L.imfcs_batch_destroy.argtypes = [vp]
    L.imfcs_batch_execute.argtypes = [vp, vp, C.POINTER(Outputs), vp]
    L.imfcs_batch_synchronize.argtypes = [vp, vp]
    L.imfcs_batch_autotune.argtypes = [vp, vp, C.POINTER(Outputs), vp, C.c_int, C.POINTER(C.c_float)]
    L.imfcs_batch_job_info.argtypes = [vp, C.c_int, ip, ip, ip, ip, ip, ip, C.POINTER(C.c_float)]
    L.imfcs_batch_lanes.argtypes = [vp]
    L.imfcs_batch_scratch_bytes.restype = C.c_size_t
    L.imfcs_batch_scratch_bytes.argtypes = [vp]
    L.imfcs_batch_kernel_launches.argtypes = [vp]
    L.imfcs_tiff_open.argtypes = [C.c_char_p, C.POINTER(C.c_void_p), ip, ip, ip]
    L.imfcs_tiff_read.argtypes = [vp, C.c_int, C.c_int, vp]
    L.imfcs_tiff_read_device.argtypes = [vp, C.c_int, C.c_int, vp, vp]
    L.imfcs_tiff_close.argtypes = [vp]
    L.imfcs_background_stats.argtypes = [vp, C.c_int, C.c_int, C.c_int, vp, vp, vp, vp, vp, vp]
    L.imfcs_bands_create.argtypes = [C.POINTER(Config), C.c_int, C.c_size_t, C.POINTER(C.c_void_p)]
    L.imfcs_bands_destroy.argtypes = [vp]
    L.imfcs_bands_geometry.argtypes = [vp, ip, ip, C.POINTER(C.c_size_t)]
    L.imfcs_bands_plan.restype = vp
    L.imfcs_bands_plan.argtypes = [vp]
    L.imfcs_bands_execute.argtypes = [vp, vp, C.POINTER(Outputs), vp]
    L.imfcs_measure_fp32_fma_rate.argtypes = [dp, vp]
    L.imfcs_bands_set_background_image.argtypes = [vp, vp]
    L.imfcs_band_window.argtypes = [C.POINTER(Config), C.c_int, C.c_int, ip, ip, ip, ip, ip]


def load(build_if_missing: bool = True) -> C.CDLL:
    """Load the in-tree library (building it with nvcc if absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise ImfcsError(f"{LIB_PATH} is missing; run imaging_fcs_1_52_gb300.build")
        from . import build as _build
        _build.build()
    if not os.path.exists(LIB_PATH):
        raise ImfcsError(f"{LIB_PATH} could not be built")
    _lib = C.CDLL(LIB_PATH)
    _declare(_lib)
    return _lib


def last_error() -> str:
    msg = load().imfcs_get_last_error()
    return msg.decode() if msg else ""


def check(rc: int, what: str) -> None:
    if rc != 0:
        raise ImfcsError(f"{what} failed: {last_error()}")
