"""ctypes binding of libmwsep_gb300.so (the C ABI in include/milkyway_separation_gb300.h).

The structure layouts below mirror the reference's problem structs
(milkyway_separation/cpu/parameters.h:27-71, star_points.h:27-31,
evaluation_state.h:30-58); tests check ``ctypes.sizeof`` against the C side.

There is no CPU fallback: if the shared library is missing this module raises
on first use, and every compute call fails with MWSEP_ERR_CUDA on a machine
without an sm_103 GPU.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import build as _build

MWSEP_OK = 0
MWSEP_ERR_ARG = 1
MWSEP_ERR_IO = 2
MWSEP_ERR_PARAM_COUNT = 3
MWSEP_ERR_UNSUPPORTED = 4
MWSEP_ERR_CUDA = 5
MWSEP_ERR_NOMEM = 6
MWSEP_ERR_BUDGET = 7
MWSEP_ERR_TIMEOUT = 8
MWSEP_ERR_CANCELLED = 9
MWSEP_ERR_STATE = 10
MWSEP_ERR_BUSY = 11

MWSEP_MAX_STREAMS = 8
MWSEP_MAX_AREAS = 8
MWSEP_MAX_CONVOLVE = 512

MWSEP_PLAIN_F64 = 0
MWSEP_MIXED_F32 = 1
MWSEP_PLAIN_DF = 2


class INTEGRAL(C.Structure):
    _fields_ = [
        ("r_min", C.c_double), ("r_max", C.c_double), ("r_step_size", C.c_double),
        ("nu_min", C.c_double), ("nu_max", C.c_double), ("nu_step_size", C.c_double),
        ("mu_min", C.c_double), ("mu_max", C.c_double), ("mu_step_size", C.c_double),
        ("r_steps", C.c_int), ("nu_steps", C.c_int), ("mu_steps", C.c_int),
        ("min_calculation", C.c_long), ("max_calculation", C.c_long),
    ]


class ASTRONOMY_PARAMETERS(C.Structure):
    _fields_ = [
        ("parameters_version", C.c_double),
        ("number_background_parameters", C.c_int),
        ("background_weight", C.c_double),
        ("background_parameters", C.POINTER(C.c_double)),
        ("background_step", C.POINTER(C.c_double)),
        ("background_min", C.POINTER(C.c_double)),
        ("background_max", C.POINTER(C.c_double)),
        ("background_optimize", C.POINTER(C.c_int)),
        ("number_streams", C.c_int),
        ("number_stream_parameters", C.c_int),
        ("stream_weights", C.POINTER(C.c_double)),
        ("stream_weight_step", C.POINTER(C.c_double)),
        ("stream_weight_min", C.POINTER(C.c_double)),
        ("stream_weight_max", C.POINTER(C.c_double)),
        ("stream_weight_optimize", C.POINTER(C.c_int)),
        ("stream_parameters", C.POINTER(C.POINTER(C.c_double))),
        ("stream_step", C.POINTER(C.POINTER(C.c_double))),
        ("stream_min", C.POINTER(C.POINTER(C.c_double))),
        ("stream_max", C.POINTER(C.POINTER(C.c_double))),
        ("stream_optimize", C.POINTER(C.POINTER(C.c_int))),
        ("convolve", C.c_int),
        ("sgr_coordinates", C.c_int),
        ("aux_bg_profile", C.c_int),
        ("wedge", C.c_int),
        ("number_integrals", C.c_int),
        ("integral", C.POINTER(C.POINTER(INTEGRAL))),
    ]


class STAR_POINTS(C.Structure):
    _fields_ = [("number_stars", C.c_int), ("stars", C.POINTER(C.POINTER(C.c_double)))]


class INTEGRAL_AREA(C.Structure):
    _fields_ = [
        ("mu_steps", C.c_int), ("nu_steps", C.c_int), ("r_steps", C.c_int),
        ("mu_min", C.c_double), ("nu_min", C.c_double), ("r_min", C.c_double),
        ("mu_max", C.c_double), ("nu_max", C.c_double), ("r_max", C.c_double),
        ("mu_step_size", C.c_double), ("nu_step_size", C.c_double), ("r_step_size", C.c_double),
        ("min_calculation", C.c_long), ("max_calculation", C.c_long), ("current_calculation", C.c_long),
        ("number_streams", C.c_int),
        ("background_integral", C.c_double),
        ("stream_integrals", C.POINTER(C.c_double)),
    ]


class EVALUATION_STATE(C.Structure):
    _fields_ = [
        ("integral", C.POINTER(C.POINTER(INTEGRAL_AREA))),
        ("current_integral", C.c_int), ("number_streams", C.c_int), ("number_integrals", C.c_int),
        ("background_integral", C.c_double),
        ("stream_integrals", C.POINTER(C.c_double)),
        ("current_star_point", C.c_int), ("total_stars", C.c_int),
        ("num_zero", C.c_int), ("bad_jacobians", C.c_int),
        ("prob_sum", C.c_double),
    ]


class mwsep_result(C.Structure):
    _fields_ = [
        ("likelihood", C.c_double),
        ("prob_sum", C.c_double),
        ("num_zero", C.c_int),
        ("number_streams", C.c_int),
        ("number_integrals", C.c_int),
        ("status", C.c_int),
        ("background_integral", C.c_double),
        ("stream_integrals", C.c_double * MWSEP_MAX_STREAMS),
        ("area_integrals", (C.c_double * (1 + MWSEP_MAX_STREAMS)) * MWSEP_MAX_AREAS),
        ("background_only_likelihood", C.c_double),
        ("stream_only_likelihood", C.c_double * MWSEP_MAX_STREAMS),
    ]


class mwsep_pipe_peaks(C.Structure):
    _fields_ = [("fp64_fma_tflops", C.c_double), ("fp32_fma_tflops", C.c_double), ("ex2_gops", C.c_double),
                ("rsqrt_gops", C.c_double), ("rcp_gops", C.c_double), ("sm_count", C.c_int)]


class mwsep_area_tables(C.Structure):
    _fields_ = [("mu_steps", C.c_int), ("nu_steps", C.c_int), ("r_steps", C.c_int), ("convolve", C.c_int),
                ("geom", C.c_void_p), ("r_point", C.c_void_p), ("qw_r3_N", C.c_void_p),
                ("r_in_mag", C.c_void_p), ("r_in_mag2", C.c_void_p), ("reff_xr_rp3", C.c_void_p),
                ("irv", C.c_void_p), ("ids", C.c_void_p),
                ("min_calculation", C.c_long), ("max_calculation", C.c_long)]


class mwsep_density_params(C.Structure):
    _fields_ = [("alpha", C.c_double), ("q", C.c_double), ("r0", C.c_double), ("delta", C.c_double),
                ("aux_bg_profile", C.c_int), ("bg_a", C.c_double), ("bg_b", C.c_double), ("bg_c", C.c_double),
                ("number_streams", C.c_int), ("stream_sigma", C.c_double * MWSEP_MAX_STREAMS),
                ("stream_a", (C.c_double * 3) * MWSEP_MAX_STREAMS),
                ("stream_c", (C.c_double * 3) * MWSEP_MAX_STREAMS)]


MWSEP_NOALLOC_SCRATCH_BYTES = 256 * 1024


class mwsep_server_config(C.Structure):
    _fields_ = [("lanes", C.c_int), ("max_batch", C.c_int), ("lane_hbm_bytes", C.c_size_t),
                ("target_batch_ms", C.c_double), ("max_queued", C.c_longlong)]


class mwsep_server_stats(C.Structure):
    _fields_ = [("completed", C.c_longlong), ("failed", C.c_longlong), ("cancelled", C.c_longlong),
                ("batches", C.c_longlong), ("queued", C.c_longlong), ("mean_batch", C.c_double),
                ("p50_latency_s", C.c_double), ("p99_latency_s", C.c_double), ("max_latency_s", C.c_double),
                ("evals_per_s", C.c_double), ("refused", C.c_longlong), ("max_queue", C.c_longlong)]


class mwsep_request(C.Structure):
    _fields_ = [("wedge", C.c_int), ("theta", C.POINTER(C.c_double))]


class mwsep_star_catalogue(C.Structure):
    _fields_ = [("number_stars", C.c_int), ("l", C.POINTER(C.c_double)), ("b", C.POINTER(C.c_double)),
                ("r", C.POINTER(C.c_double)), ("map", C.c_void_p), ("map_bytes", C.c_size_t)]


class mwsep_separation_summary(C.Structure):
    _fields_ = [("number_streams", C.c_int), ("likelihood", C.c_double), ("background_integral", C.c_double),
                ("stream_integrals", C.c_double * MWSEP_MAX_STREAMS), ("expected", C.c_double * MWSEP_MAX_STREAMS),
                ("assigned", C.c_longlong * MWSEP_MAX_STREAMS), ("background_assigned", C.c_longlong)]

EvalFunc = C.CFUNCTYPE(C.c_double, C.POINTER(C.c_double), C.POINTER(ASTRONOMY_PARAMETERS),
                       C.POINTER(EVALUATION_STATE), C.POINTER(STAR_POINTS))

_P = C.POINTER
_SIGS = {
    "mwsep_status_string": (C.c_char_p, [C.c_int]),
    "mwsep_last_error": (C.c_int, []),
    "mwsep_version": (C.c_char_p, []),
    "mwsep_device_checks": (C.c_int, [C.c_int, _P(C.c_int), _P(C.c_ulonglong), _P(C.c_ulonglong)]),
    "mwsep_df_eval": (C.c_int, [C.c_int, C.c_int, C.c_int, _P(C.c_double), _P(C.c_double), _P(C.c_double),
                                _P(C.c_double)]),
    "mwsep_log10_sum_eval": (C.c_int, [C.c_int, C.c_int, _P(C.c_double), _P(C.c_double)]),
    "mwsep_read_astronomy_parameters": (C.c_int, [C.c_char_p, _P(ASTRONOMY_PARAMETERS)]),
    "mwsep_write_astronomy_parameters": (C.c_int, [C.c_char_p, _P(ASTRONOMY_PARAMETERS)]),
    "mwsep_free_parameters": (None, [_P(ASTRONOMY_PARAMETERS)]),
    "mwsep_get_optimized_parameter_count": (C.c_int, [_P(ASTRONOMY_PARAMETERS)]),
    "mwsep_set_astronomy_parameters": (C.c_int, [_P(ASTRONOMY_PARAMETERS), _P(C.c_double)]),
    "mwsep_get_search_parameters": (C.c_int, [_P(ASTRONOMY_PARAMETERS), _P(C.c_double)]),
    "mwsep_split_astronomy_parameters": (C.c_int, [_P(ASTRONOMY_PARAMETERS), C.c_int, C.c_int]),
    "mwsep_read_star_points": (C.c_int, [C.c_char_p, _P(STAR_POINTS)]),
    "mwsep_write_star_points": (C.c_int, [C.c_char_p, _P(STAR_POINTS)]),
    "mwsep_free_star_points": (None, [_P(STAR_POINTS)]),
    "mwsep_split_star_points": (C.c_int, [_P(STAR_POINTS), C.c_int, C.c_int]),
    "mwsep_initialize_state": (C.c_int, [_P(ASTRONOMY_PARAMETERS), _P(STAR_POINTS), _P(EVALUATION_STATE)]),
    "mwsep_free_state": (None, [_P(EVALUATION_STATE)]),
    "mwsep_evaluate": (C.c_double, [_P(C.c_double), _P(ASTRONOMY_PARAMETERS), _P(EVALUATION_STATE),
                                    _P(STAR_POINTS)]),
    "mwsep_evaluate_mixed": (C.c_double, [_P(C.c_double), _P(ASTRONOMY_PARAMETERS),
                                          _P(EVALUATION_STATE), _P(STAR_POINTS)]),
    "mwsep_evaluate_df": (C.c_double, [_P(C.c_double), _P(ASTRONOMY_PARAMETERS),
                                       _P(EVALUATION_STATE), _P(STAR_POINTS)]),
    "mwsep_ctx_create": (C.c_int, [C.c_int, _P(C.c_void_p)]),
    "mwsep_ctx_destroy": (C.c_int, [C.c_void_p]),
    "mwsep_ctx_set_problem": (C.c_int, [C.c_void_p, _P(ASTRONOMY_PARAMETERS)]),
    "mwsep_ctx_set_stars": (C.c_int, [C.c_void_p, _P(STAR_POINTS)]),
    "mwsep_ctx_set_stars_soa": (C.c_int, [C.c_void_p, C.c_int, _P(C.c_double), _P(C.c_double),
                                          _P(C.c_double)]),
    "mwsep_ctx_theta_count": (C.c_int, [C.c_void_p]),
    "mwsep_ctx_evaluate": (C.c_int, [C.c_void_p, _P(C.c_double), C.c_int, _P(mwsep_result)]),
    "mwsep_ctx_integrals": (C.c_int, [C.c_void_p, _P(C.c_double), C.c_int, _P(mwsep_result)]),
    "mwsep_ctx_likelihood": (C.c_int, [C.c_void_p, _P(C.c_double), _P(C.c_double), C.c_int, _P(mwsep_result)]),
    "mwsep_integral_f": (None, [_P(C.c_double), _P(C.c_double), _P(ASTRONOMY_PARAMETERS), _P(EVALUATION_STATE),
                                _P(STAR_POINTS)]),
    "mwsep_likelihood_f": (None, [_P(C.c_double), _P(C.c_double), _P(ASTRONOMY_PARAMETERS), _P(EVALUATION_STATE),
                                  _P(STAR_POINTS)]),
    "mwsep_ctx_evaluate_batch": (C.c_int, [C.c_void_p, C.c_int, _P(C.c_double), C.c_int,
                                           _P(mwsep_result)]),
    "mwsep_ctx_device_bytes": (C.c_int, [C.c_void_p, _P(C.c_size_t)]),
    "mwsep_ctx_last_timings": (C.c_int, [C.c_void_p, _P(C.c_double)]),
    "mwsep_ctx_last_launches": (C.c_int, [C.c_void_p, _P(C.c_int)]),
    "mwsep_ctx_transfer_bytes": (C.c_int, [C.c_void_p, _P(C.c_size_t), _P(C.c_size_t)]),
    "mwsep_ctx_separation": (C.c_int, [C.c_void_p, _P(C.c_double), C.c_ulonglong, _P(C.c_double), _P(C.c_int),
                                       _P(C.c_double), _P(mwsep_separation_summary)]),
    "mwsep_stripe_transform": (C.c_int, [C.c_int, C.c_int, _P(C.c_double)]),
    "mwsep_write_separation": (C.c_int, [C.c_char_p, C.c_int, _P(C.c_int), _P(C.c_double)]),
    "mwsep_get_step": (C.c_int, [_P(ASTRONOMY_PARAMETERS), _P(C.c_double)]),
    "mwsep_write_star_catalogue": (C.c_int, [C.c_char_p, C.c_int, _P(C.c_double), _P(C.c_double),
                                             _P(C.c_double)]),
    "mwsep_write_star_points_binary": (C.c_int, [C.c_char_p, _P(STAR_POINTS)]),
    "mwsep_map_star_catalogue": (C.c_int, [C.c_char_p, _P(mwsep_star_catalogue)]),
    "mwsep_unmap_star_catalogue": (C.c_int, [_P(mwsep_star_catalogue)]),
    "mwsep_read_star_points_binary": (C.c_int, [C.c_char_p, _P(STAR_POINTS)]),
    "mwsep_write_astronomy_parameters_binary": (C.c_int, [C.c_char_p, _P(ASTRONOMY_PARAMETERS)]),
    "mwsep_read_astronomy_parameters_binary": (C.c_int, [C.c_char_p, _P(ASTRONOMY_PARAMETERS)]),
    "mwsep_ctx_set_stars_file": (C.c_int, [C.c_void_p, C.c_char_p]),
    "mwsep_get_min_parameters": (C.c_int, [_P(ASTRONOMY_PARAMETERS), _P(C.c_double)]),
    "mwsep_get_max_parameters": (C.c_int, [_P(ASTRONOMY_PARAMETERS), _P(C.c_double)]),
    "mwsep_ctx_gradient": (C.c_int, [C.c_void_p, C.c_int, _P(C.c_double), _P(C.c_double), C.c_int,
                                     _P(C.c_double), _P(C.c_double)]),
    "mwsep_ctx_hessian": (C.c_int, [C.c_void_p, C.c_int, _P(C.c_double), _P(C.c_double), C.c_int,
                                    _P(C.c_double), _P(C.c_double), _P(C.c_double)]),
    "mwsep_invert_matrix": (C.c_int, [C.c_int, _P(C.c_double), _P(C.c_double)]),
    "mwsep_errors_from_hessian": (C.c_int, [C.c_int, _P(C.c_double), C.c_int, _P(C.c_double),
                                            _P(C.c_double)]),
    "mwsep_write_errors": (C.c_int, [C.c_char_p, C.c_int, _P(C.c_double), _P(C.c_double), _P(C.c_double)]),
    "mwsep_ctx_add_wedge": (C.c_int, [C.c_void_p, _P(ASTRONOMY_PARAMETERS), _P(STAR_POINTS), _P(C.c_int)]),
    "mwsep_ctx_wedge_theta_count": (C.c_int, [C.c_void_p, C.c_int]),
    "mwsep_ctx_wedge_bytes": (C.c_int, [C.c_void_p, C.c_int, _P(C.c_size_t)]),
    "mwsep_ctx_wedge_points": (C.c_int, [C.c_void_p, C.c_int, _P(C.c_double)]),
    "mwsep_ctx_set_hbm_budget": (C.c_int, [C.c_void_p, C.c_size_t]),
    "mwsep_ctx_evaluate_requests": (C.c_int, [C.c_void_p, C.c_int, _P(mwsep_request), C.c_int,
                                              _P(mwsep_result)]),
    "mwsep_ctx_autotune": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _P(C.c_double)]),
    "mwsep_ctx_wedge_tile_shape": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _P(C.c_int), _P(C.c_int)]),
    "mwsep_model_tile_cost": (C.c_double, [C.c_int, C.c_int, C.c_int, C.c_longlong, C.c_int, C.c_int, C.c_int,
                                           C.c_int, C.c_double]),
    "mwsep_model_kchunk": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_longlong, C.c_longlong, C.c_int, C.c_int,
                                     _P(C.c_int), _P(C.c_double)]),
    "mwsep_server_create": (C.c_int, [C.c_void_p, _P(mwsep_server_config), _P(C.c_void_p)]),
    "mwsep_server_submit": (C.c_int, [C.c_void_p, C.c_int, _P(C.c_double), C.c_int, _P(C.c_ulonglong)]),
    "mwsep_server_wait": (C.c_int, [C.c_void_p, C.c_ulonglong, C.c_double, _P(mwsep_result)]),
    "mwsep_server_cancel": (C.c_int, [C.c_void_p, C.c_ulonglong]),
    "mwsep_server_get_stats": (C.c_int, [C.c_void_p, _P(mwsep_server_stats)]),
    "mwsep_server_reset_stats": (C.c_int, [C.c_void_p]),
    "mwsep_server_destroy": (C.c_int, [C.c_void_p]),
    "mwsep_evalfunc_transfer_bytes": (C.c_int, [_P(C.c_size_t), _P(C.c_size_t)]),
    "mwsep_measure_pipe_peaks": (C.c_int, [C.c_int, _P(mwsep_pipe_peaks)]),
    "mwsep_area_integrals_noalloc": (C.c_int, [_P(mwsep_area_tables), _P(mwsep_density_params), C.c_void_p,
                                               C.c_void_p]),
}

_lib = None
_lock = threading.Lock()


def library_path() -> str:
    """The in-tree library, or MWSEP_LIBRARY when set (a variant build)."""
    return os.environ.get("MWSEP_LIBRARY") or _build.LIB_PATH


def lib(build_if_missing: bool = False):
    """Load libmwsep_gb300.so.  Raises if it is missing (no fallback)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = library_path()
        if not os.path.exists(path):
            if not build_if_missing:
                raise RuntimeError(f"{path} is missing: build it with "
                                   "`python -c 'import __graft_entry__ as g; g.build()'`")
            _build.build()
        L = C.CDLL(path)
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
        return _lib


def exported_symbols():
    return list(_SIGS.keys())


class MwsepError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        msg = lib().mwsep_status_string(status).decode()
        super().__init__(f"{what}: {msg} (status {status})" if what else msg)


def check(status: int, what: str = "") -> None:
    if status != MWSEP_OK:
        raise MwsepError(status, what)
