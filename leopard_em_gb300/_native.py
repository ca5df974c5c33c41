"""ctypes binding of the C ABI in ``include/leopard_gb300.h``.

The library is the in-tree ``_build/libleopard_gb300.so`` produced by
``leopard_em_gb300.build``.  There is no fallback: if the library is missing
or a call fails, a RuntimeError (ValueError for bad arguments) is raised.
"""

from __future__ import annotations

import ctypes
import os
import threading

from . import build as _build

_LOCK = threading.Lock()
_LIB = None

LGB_OK = 0
LGB_ERR_INVALID_ARGUMENT = 1
LGB_ERR_UNSUPPORTED_SIZE = 2
LGB_ERR_WORKSPACE_TOO_SMALL = 3
LGB_ERR_CUDA = 4
LGB_ERR_DEVICE_TIMEOUT = 5


class MatchProblem(ctypes.Structure):
    """Mirror of ``lgb_match_problem``."""

    _fields_ = [
        ("image_h", ctypes.c_int),
        ("image_w", ctypes.c_int),
        ("template_size", ctypes.c_int),
        ("n_pixel_sizes", ctypes.c_int),
        ("n_defocus", ctypes.c_int),
        ("n_orientations", ctypes.c_int),
        ("orientation_batch", ctypes.c_int),
        ("micrograph_h", ctypes.c_int),  # 0 = image_h (no zero padding)
        ("micrograph_w", ctypes.c_int),  # 0 = image_w
        ("col_waves", ctypes.c_int),  # 0 = default column-pass launch shape
    ]


class RefineProblem(ctypes.Structure):
    """Mirror of ``lgb_refine_problem``."""

    _fields_ = [
        ("image_h", ctypes.c_int),
        ("image_w", ctypes.c_int),
        ("template_size", ctypes.c_int),
        ("n_pixel_sizes", ctypes.c_int),
        ("n_defocus", ctypes.c_int),
        ("n_offsets", ctypes.c_int),
        ("offset_batch", ctypes.c_int),
        ("n_particles", ctypes.c_int),
    ]


class CtfParams(ctypes.Structure):
    """Mirror of ``lgb_ctf_params``."""

    _fields_ = [
        ("voltage_kv", ctypes.c_double),
        ("spherical_aberration_mm", ctypes.c_double),
        ("amplitude_contrast", ctypes.c_double),
        ("b_factor", ctypes.c_double),
        ("phase_shift_deg", ctypes.c_double),
        ("pixel_size", ctypes.c_double),
    ]


_P = ctypes.c_void_p
_I = ctypes.c_int
_LL = ctypes.c_longlong
_SZ = ctypes.c_size_t
_PROB = ctypes.POINTER(MatchProblem)

_SIGNATURES = {
    "lgb_status_string": ([_I], ctypes.c_char_p),
    "lgb_version": ([], _I),
    "lgb_profile_begin": ([], _I),
    "lgb_profile_end": ([ctypes.POINTER(ctypes.c_double), ctypes.POINTER(_LL), _I], _I),
    "lgb_match_supported": ([_PROB], _I),
    "lgb_match_workspace_size": ([_PROB, ctypes.POINTER(_SZ)], _I),
    "lgb_match_init_stats": ([_LL, _P, _P, _P, _P, _P], _I),
    "lgb_match_prepare_image": ([_PROB, _P, _P, _SZ, _P], _I),
    "lgb_match_filters": ([_PROB, _P, _P, _P, _P], _I),
    "lgb_match_search": ([_PROB, _P, _P, _P, _I, _I, _P, _P, _P, _P, _P, _SZ, _P], _I),
    "lgb_match_fft_size": ([_I, _I], _I),
    "lgb_match_search_graph": ([_PROB, _P, _P, _P, _I, _I, _I, _P, _P, _P, _P, _P, _SZ, _P], _I),
    "lgb_match_plan_create": ([_PROB, ctypes.POINTER(_I)], _P),
    "lgb_match_plan_destroy": ([_P], None),
    "lgb_match_plan_set_filters": ([_P, _P, _P, _P], _I),
    "lgb_match_plan_set_image": ([_P, _P, _P], _I),
    "lgb_match_plan_search": ([_P, _P, _P, _I, _I, _P], _I),
    "lgb_match_plan_maps": ([_P] + [ctypes.POINTER(_P)] * 4, _I),
    "lgb_match_plan_finalize": ([_P] + [_P] * 9 + [_P], _I),
    "lgb_static_scratch_capacity": ([], _SZ),
    "lgb_match_search_static_scratch": ([_PROB, _P, _P, _P, _P, _I, _I, _P, _P, _P, _P, _P], _I),
    "lgb_refine_supported": ([ctypes.POINTER(RefineProblem)], _I),
    "lgb_refine_workspace_size": ([ctypes.POINTER(RefineProblem), ctypes.POINTER(_SZ)], _I),
    "lgb_refine_search": ([ctypes.POINTER(RefineProblem), ctypes.POINTER(CtfParams)] + [_P] * 18 + [_SZ, _P], _I),
    "lgb_match_precision_supported": ([_PROB, _I], _I),
    "lgb_match_precision_workspace_size": ([_PROB, ctypes.POINTER(_SZ)], _I),
    "lgb_match_search_precision": ([_PROB, _I, _P, _P, _P, _I, _I, _P, _P, _P, _P, _P, _SZ, _P, _P], _I),
    "lgb_xcorr_stack_supported": ([_I, _I, _I], _I),
    "lgb_xcorr_stack_workspace_size": ([_I, _I, _I, _I, _I, ctypes.POINTER(_SZ)], _I),
    "lgb_xcorr_stack": ([_I] * 6 + [_P] * 6 + [_SZ, _P], _I),
    "lgb_peaks_scratch_size": ([_I, _I, _I], _SZ),
    "lgb_peaks_find": ([_I, _I, _P, ctypes.c_float, ctypes.c_float, _I, _P, _SZ, _I, _P,
                        ctypes.POINTER(_I), ctypes.POINTER(_I), _P], _I),
    "lgb_wait_timeout_selftest": ([ctypes.c_uint, _P, _P], _I),
    "lgb_ctf_filter_stack": ([_I, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.POINTER(CtfParams), _P, _I,
                              _P, _I, _P, _P], _I),
    "lgb_radial_spectrum": ([_I, _I, _I, _P, _I, ctypes.c_double, _I, _P, _P, _P], _I),
    "lgb_whitening_filter": ([_I, _I, ctypes.c_double, _I, _P, _P, _I, _I, _P, _P], _I),
    "lgb_bandpass_filter": ([_I, _I, ctypes.c_double, ctypes.c_double, ctypes.c_double, _P, _P], _I),
    "lgb_preprocess_image": ([_I, _I, _I, _P, _P, _LL, _P, ctypes.c_double, _P, _P, _P], _I),
    "lgb_tc_gemm": ([_I] * 6 + [_P] * 5 + [_I, _I, _I, _P, _P], _I),
    "lgb_nn_conv3x3_workspace_size": ([_I] * 6 + [ctypes.POINTER(_SZ)], _I),
    "lgb_nn_conv3x3_forward": ([_I] * 7 + [_P] * 5 + [_SZ, _P, _P], _I),
    "lgb_nn_conv3x3_backward": ([_I] * 6 + [_P] * 7 + [_SZ, _P, _P], _I),
    "lgb_nn_linear_workspace_size": ([_I] * 3 + [ctypes.POINTER(_SZ)], _I),
    "lgb_nn_linear_forward": ([_I] * 4 + [_P] * 6 + [_SZ, _P, _P], _I),
    "lgb_nn_linear_backward": ([_I] * 3 + [_P] * 7 + [_SZ, _P, _P], _I),
    "lgb_nn_relu_backward": ([_LL, _P, _P, _P, _P], _I),
    "lgb_nn_mse": ([_I, _I] + [_P] * 5 + [_P], _I),
    "lgb_nn_adam": ([_LL] + [_P] * 5 + [ctypes.c_float] * 5 + [_I, _P], _I),
    "lgb_nn_to_bf16": ([_LL, _P, _P, _P], _I),
    "lgb_nn_make_inputs": ([_I, _I, _I, _P, _P, _I] + [_P] * 4 + [ctypes.POINTER(CtfParams), _I, _I, _P, _P], _I),
    "lgb_nn_gauss_newton": ([_I, _I, _I, _P, _P, _P], _I),
    "lgb_match_finalize": ([_PROB, _LL, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P], _I),
}


STAGE_NAMES = ("slice", "proj_col", "proj_row", "pad_rfft", "colpass", "rowpass", "colfwd", "dft_col_gemm",
               "dft_row_gemm")


class StageProfile:
    """Context manager: per-stage device time (ms) and launch counts of every
    search or refinement call made inside the ``with`` block."""

    def __enter__(self):
        check(lib().lgb_profile_begin(), "lgb_profile_begin")
        self.ms = {}
        self.launches = {}
        return self

    def __exit__(self, *exc):
        n = len(STAGE_NAMES)
        ms = (ctypes.c_double * n)()
        cnt = (_LL * n)()
        check(lib().lgb_profile_end(ms, cnt, n), "lgb_profile_end")
        self.ms = {k: ms[i] for i, k in enumerate(STAGE_NAMES)}
        self.launches = {k: int(cnt[i]) for i, k in enumerate(STAGE_NAMES)}
        return False


def library_path() -> str:
    return _build.LIB_PATH


def lib():
    """Load (once) and return the CUDA library; raise if it was never built."""
    global _LIB
    with _LOCK:
        if _LIB is None:
            path = library_path()
            if not os.path.exists(path):
                raise RuntimeError(
                    f"leopard_em_gb300 CUDA library not found at {path}; build it with "
                    "`python -m leopard_em_gb300.build` (there is no CPU fallback)"
                )
            handle = ctypes.CDLL(path)
            for name, (args, res) in _SIGNATURES.items():
                fn = getattr(handle, name)
                fn.argtypes = args
                fn.restype = res
            _LIB = handle
    return _LIB


def check(status: int, what: str) -> None:
    """Turn a non-zero lgb_status into a Python exception."""
    if status == LGB_OK:
        return
    msg = lib().lgb_status_string(status).decode()
    if status in (LGB_ERR_INVALID_ARGUMENT, LGB_ERR_UNSUPPORTED_SIZE, LGB_ERR_WORKSPACE_TOO_SMALL):
        raise ValueError(f"{what}: {msg} (status {status})")
    raise RuntimeError(f"{what}: {msg} (status {status})")
