"""ctypes declarations of the C ABI in include/rdxg.h (libredux_gb300.so)."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libredux_gb300.so")

RDXG_OK, RDXG_ERR_ARG, RDXG_ERR_UNSUPPORTED, RDXG_ERR_CUDA, RDXG_ERR_STATE, RDXG_ERR_NONFINITE, RDXG_ERR_NOMEM = range(7)
RDXG_FP32, RDXG_FP64 = 0, 1
RDXG_GRAD_VOGEL, RDXG_GRAD_EXACT, RDXG_GRAD_FD = 0, 1, 2
RDXG_RESTORE_PSF, RDXG_RESTORE_PSF_AVG, RDXG_RESTORE_COBJ, RDXG_RESTORE_RESIDUAL = 1, 2, 4, 8

EXPORTED = ("rdxg_version", "rdxg_create", "rdxg_destroy", "rdxg_last_error", "rdxg_set_stream",
            "rdxg_set_patches", "rdxg_set_patches_device", "rdxg_metric", "rdxg_gradient",
            "rdxg_solve", "rdxg_solve_async", "rdxg_solve_many", "rdxg_fetch_results", "rdxg_last_launch_count",
            "rdxg_debug_copy", "rdxg_cg_minimize", "rdxg_profile_kernels", "rdxg_metric_with_reference",
            "rdxg_metric_noalloc", "rdxg_restore", "rdxg_restore_ex", "rdxg_set_phase_mode", "rdxg_phase_mode",
            "rdxg_autotune", "rdxg_set_launch_shape", "rdxg_get_launch_shape", "rdxg_set_fit_plane",
            "rdxg_set_initial_alpha", "rdxg_set_reg_alpha", "rdxg_debug_set", "rdxg_set_start_alpha",
            "rdxg_set_recompute", "rdxg_recompute", "rdxg_pupil_size", "rdxg_make_pupil", "rdxg_pupil_support",
            "rdxg_make_modes", "rdxg_apodization_windows", "rdxg_set_patch_shapes")


class Geometry(C.Structure):
    _fields_ = [(n, C.c_int32) for n in (
        "otf_size", "pupil_pixels", "patch_size", "n_modes", "n_objects", "n_images", "n_channels",
        "tilt_x", "tilt_y", "n_free", "cutout_size", "max_patches", "precision", "device", "eval_chunk")]


class Static(C.Structure):
    _fields_ = [("modes", C.c_void_p), ("pupil", C.c_void_p),
                ("n_pupil_support", C.c_int32), ("pupil_support", C.c_void_p),
                ("n_otf_support", C.c_int32), ("otf_support", C.c_void_p),
                ("image_object", C.c_void_p), ("image_channel", C.c_void_p),
                ("phi_fixed", C.c_void_p), ("object_weight", C.c_void_p),
                ("object_grad_step", C.c_void_p), ("window", C.c_void_p), ("noise_window", C.c_void_p),
                ("ns_nnz", C.c_int64), ("ns_rows", C.c_void_p), ("ns_cols", C.c_void_p),
                ("ns_vals", C.c_void_p), ("tilt_jacobian", C.c_void_p)]


class SolveParams(C.Structure):
    _fields_ = [("mode_start", C.c_int32), ("mode_step", C.c_int32), ("max_iterations", C.c_int32),
                ("min_iterations", C.c_int32), ("target_iterations", C.c_int32), ("fd_first", C.c_int32),
                ("max_metrics", C.c_int32), ("check_every", C.c_int32), ("ftol", C.c_double),
                ("eps", C.c_double)]


class PatchShape(C.Structure):
    _fields_ = [("frames", C.c_int32), ("n_modes", C.c_int32), ("n_free", C.c_int32), ("ns_nnz", C.c_int64),
                ("ns_rows", C.c_void_p), ("ns_cols", C.c_void_p), ("ns_vals", C.c_void_p)]


class ModeParams(C.Structure):
    _fields_ = [("kind", C.c_int32), ("pupil_pixels", C.c_int32), ("radius", C.c_double),
                ("wavelength", C.c_double), ("angle", C.c_double), ("jacobian_scale", C.c_double),
                ("kl_first", C.c_int32), ("kl_last", C.c_int32), ("kl_cutoff", C.c_double)]


class LaunchShape(C.Structure):
    _fields_ = [("eval_threads", C.c_int32), ("forward_threads", C.c_int32), ("adjoint_threads", C.c_int32),
                ("eval_radix", C.c_int32), ("forward_radix", C.c_int32), ("adjoint_radix", C.c_int32),
                ("solver_form", C.c_int32)]


class PatchReport(C.Structure):
    _fields_ = [("initial_metric", C.c_double), ("final_metric", C.c_double), ("iterations", C.c_int32),
                ("status", C.c_int32), ("n_f_evals", C.c_int32), ("n_df_evals", C.c_int32),
                ("fail_count", C.c_int32), ("n_metrics", C.c_int32)]


F_FN = C.CFUNCTYPE(C.c_double, C.POINTER(C.c_double), C.c_void_p)
DF_FN = C.CFUNCTYPE(None, C.POINTER(C.c_double), C.c_int32, C.c_int32, C.POINTER(C.c_double), C.c_void_p)
SHIFT_FN = C.CFUNCTYPE(None, C.POINTER(C.c_double), C.c_void_p)

_LIB = None


def load(path: str = LIB_PATH):
    """Loads the library; raises if it has not been built (there is no fallback)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: run redux_gb300.build.build() first "
                           "(the solver has no CPU fallback)")
    L = C.CDLL(path)
    vp = C.c_void_p
    L.rdxg_version.restype = C.c_int
    L.rdxg_create.argtypes = [C.POINTER(Geometry), C.POINTER(Static), C.POINTER(vp)]
    L.rdxg_destroy.argtypes = [vp]
    L.rdxg_last_error.restype = C.c_char_p
    L.rdxg_last_error.argtypes = [vp]
    L.rdxg_set_stream.argtypes = [vp, vp]
    L.rdxg_set_fit_plane.argtypes = [vp, C.c_int32]
    L.rdxg_set_initial_alpha.argtypes = [vp, vp]
    L.rdxg_set_start_alpha.argtypes = [vp, vp]
    L.rdxg_set_recompute.argtypes = [vp, C.c_int32]
    L.rdxg_recompute.restype = C.c_int32
    L.rdxg_recompute.argtypes = [vp]
    L.rdxg_set_reg_alpha.argtypes = [vp, vp]
    L.rdxg_set_patches.argtypes = [vp, C.c_int32, vp, vp, vp]
    L.rdxg_set_patches_device.argtypes = [vp, C.c_int32, vp, vp, vp]
    L.rdxg_metric.argtypes = [vp, vp, vp]
    L.rdxg_metric_with_reference.argtypes = [vp, vp, vp, vp]
    L.rdxg_metric_noalloc.argtypes = [vp, vp, vp]
    L.rdxg_restore.argtypes = [vp, vp, vp, C.c_int32, vp]
    L.rdxg_restore_ex.argtypes = [vp, vp, vp, C.c_int32, C.c_int32, vp, vp, vp, vp]
    L.rdxg_gradient.argtypes = [vp, vp, vp, C.c_int32, vp, vp]
    L.rdxg_solve.argtypes = [vp, C.POINTER(SolveParams), vp, vp, vp]
    L.rdxg_solve_async.argtypes = [vp, C.POINTER(SolveParams)]
    L.rdxg_solve_many.argtypes = [C.POINTER(vp), C.c_int32, C.POINTER(SolveParams)]
    L.rdxg_fetch_results.argtypes = [vp, vp, vp, vp]
    L.rdxg_last_launch_count.restype = C.c_int64
    L.rdxg_last_launch_count.argtypes = [vp]
    L.rdxg_debug_copy.argtypes = [vp, C.c_int32, vp, C.c_size_t]
    L.rdxg_debug_set.argtypes = [vp, C.c_int32, vp, C.c_size_t]
    L.rdxg_set_phase_mode.argtypes = [vp, C.c_int32]
    L.rdxg_phase_mode.restype = C.c_int32
    L.rdxg_phase_mode.argtypes = [vp]
    L.rdxg_profile_kernels.argtypes = [vp, C.c_int32, vp]
    L.rdxg_autotune.argtypes = [vp, C.c_int32, C.POINTER(LaunchShape), vp]
    L.rdxg_set_launch_shape.argtypes = [vp, C.POINTER(LaunchShape)]
    L.rdxg_get_launch_shape.argtypes = [vp, C.POINTER(LaunchShape)]
    L.rdxg_cg_minimize.argtypes = [C.c_int32, C.c_int32, C.POINTER(SolveParams), C.c_double, F_FN, DF_FN,
                                   SHIFT_FN, vp, vp, C.POINTER(PatchReport), vp]
    L.rdxg_set_patch_shapes.argtypes = [vp, C.c_int32, C.POINTER(PatchShape), C.c_int32, vp]
    L.rdxg_pupil_size.argtypes = [C.c_int32, C.c_double, C.c_double, C.c_double, vp, vp, vp]
    L.rdxg_make_pupil.argtypes = [C.c_int32, C.c_double, C.c_double, vp, vp]
    L.rdxg_pupil_support.argtypes = [vp, C.c_int32, C.c_double, vp, vp, vp, vp, vp, vp]
    L.rdxg_make_modes.argtypes = [C.POINTER(ModeParams), vp, C.c_int32, vp, vp, vp]
    L.rdxg_apodization_windows.argtypes = [C.c_int32, C.c_int32, vp, vp]
    _LIB = L
    return L


def ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)
