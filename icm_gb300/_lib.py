"""ctypes declarations of libicm_gb300.so (the C ABI in include/*.h)."""
from __future__ import annotations

import ctypes
import os

PKG = os.path.dirname(os.path.abspath(__file__))
LIBNAME = "libicm_gb300.so"


class ICMError(Exception):
    """Raised when the GB300 library cannot be loaded or a computation fails."""


class IcmGpuOptions(ctypes.Structure):
    _fields_ = [("device_id", ctypes.c_int), ("use_cufftdx", ctypes.c_int), ("enable_graphs", ctypes.c_int),
                ("enable_q_pipeline", ctypes.c_int), ("memory_strategy", ctypes.c_int),
                ("force_uncached_fused_levels", ctypes.c_int), ("force_uncached_cufft_levels", ctypes.c_int),
                ("fast_mode", ctypes.c_int), ("verbose", ctypes.c_int)]


class IcmGpuRunStats(ctypes.Structure):
    _fields_ = [("total_ns", ctypes.c_double), ("sort_ns", ctypes.c_double),
                ("quadrature_overhead_ns", ctypes.c_double), ("block_build_ns", ctypes.c_double),
                ("tree_build_ns", ctypes.c_double), ("tree_propagate_cached_ns", ctypes.c_double),
                ("tree_propagate_recomputed_ns", ctypes.c_double), ("leaf_extract_ns", ctypes.c_double),
                ("peak_vram_bytes", ctypes.c_size_t), ("engine", ctypes.c_int), ("B", ctypes.c_int),
                ("uncached_fused_levels", ctypes.c_int), ("uncached_cufft_levels", ctypes.c_int)]


class IcmGpuPlanSummary(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int), ("k", ctypes.c_int), ("B", ctypes.c_int), ("engine", ctypes.c_int),
                ("n_levels", ctypes.c_int), ("n_tier1", ctypes.c_int), ("n_tier2", ctypes.c_int),
                ("n_tier3", ctypes.c_int), ("q_batch", ctypes.c_int),
                ("planned_peak_vram_bytes", ctypes.c_size_t)]


class IcmGb300Config(ctypes.Structure):
    _fields_ = [("block_size", ctypes.c_int), ("fft_min_degree", ctypes.c_int), ("q_chunk", ctypes.c_int),
                ("coefficient_fft_only", ctypes.c_int), ("max_device_bytes", ctypes.c_size_t),
                ("disable_zero_prefix", ctypes.c_int), ("enable_subtree", ctypes.c_int),
                ("small_max_n", ctypes.c_int), ("engine", ctypes.c_int), ("quadrature", ctypes.c_int),
                ("chunk_streams", ctypes.c_int), ("cta_points", ctypes.c_int),
                ("disable_tma", ctypes.c_int), ("vjp_spectral_min_degree", ctypes.c_int)]


_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_vp = ctypes.c_void_p

# name -> (restype, argtypes)
SIGNATURES = {
    "icm_init": (None, [ctypes.c_char_p]),
    "icm_equity": (None, [ctypes.c_int, _dp, ctypes.c_int, _dp, ctypes.c_int, _dp]),
    "icm_equity_subset": (None, [ctypes.c_int, _dp, ctypes.c_int, _dp, ctypes.c_int, _dp, _ip, ctypes.c_int]),
    "icm_select_engine": (ctypes.c_int, [ctypes.c_int, ctypes.c_int]),
    "icm_select_best_B": (ctypes.c_int, [ctypes.c_int, ctypes.c_int]),
    "icm_v1_exact": (None, [ctypes.c_int, _dp, _dp]),
    "icm_v2_exact": (None, [ctypes.c_int, _dp, _dp]),
    "icm_gpu_init": (ctypes.c_int, [ctypes.c_int]),
    "icm_gpu_shutdown": (None, []),
    "icm_gpu_last_error": (ctypes.c_char_p, []),
    "icm_gpu_release_pooled_memory": (ctypes.c_int, []),
    "icm_gpu_plan_create": (_vp, [ctypes.c_int, _dp, ctypes.c_int, ctypes.POINTER(IcmGpuOptions)]),
    "icm_gpu_plan_destroy": (None, [_vp]),
    "icm_gpu_plan_summary": (ctypes.c_int, [_vp, ctypes.POINTER(IcmGpuPlanSummary)]),
    "icm_gpu_equity_with_plan": (ctypes.c_int, [_vp, ctypes.c_int, _dp, _dp, ctypes.POINTER(IcmGpuRunStats)]),
    "icm_gb300_plan_set_targets": (ctypes.c_int, [_vp, _ip, ctypes.c_int]),
    "icm_gb300_node_work": (ctypes.c_int, [ctypes.c_int, _dp, ctypes.c_int, _ip]),
    "icm_gb300_tma_launch_count": (ctypes.c_long, []),
    "icm_gb300_current_device": (ctypes.c_int, [_ip]),
    "icm_gb300_plan_equity_dev": (ctypes.c_int, [_vp, ctypes.c_int, _vp, _vp, _vp]),
    "icm_gb300_vjp_run_dev": (ctypes.c_int, [_vp, ctypes.c_int, _vp, _vp, _vp, _vp, ctypes.c_int, _vp]),
    "icm_gb300_plan_equity_nodes": (ctypes.c_int, [_vp, ctypes.c_int, _dp, ctypes.c_int, ctypes.c_int, _dp,
                                                   ctypes.POINTER(IcmGpuRunStats)]),
    "icm_gpu_equity": (ctypes.c_int, [ctypes.c_int, _dp, ctypes.c_int, _dp, ctypes.c_int, _dp,
                                      ctypes.POINTER(IcmGpuOptions), ctypes.POINTER(IcmGpuRunStats)]),
    "icm_gpu_equity_subset": (ctypes.c_int, [ctypes.c_int, _dp, ctypes.c_int, _dp, ctypes.c_int, _dp, _ip,
                                             ctypes.c_int, ctypes.POINTER(IcmGpuOptions),
                                             ctypes.POINTER(IcmGpuRunStats)]),
    "icm_gpu_measure_hbm_bandwidth_gbps": (ctypes.c_int, [_dp]),
    "icm_gpu_measure_fused_pair_ns": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp, _dp]),
    "icm_gpu_measure_fused_r2c_pair_ns": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp, _dp]),
    "icm_last_status": (ctypes.c_int, []),
    "icm_gb300_set_config": (ctypes.c_int, [ctypes.POINTER(IcmGb300Config)]),
    "icm_gb300_player_order": (ctypes.c_int, [ctypes.c_int, _dp, _ip]),
    "icm_gb300_test_fail_allocation": (None, [ctypes.c_int]),
    "icm_gb300_check_geometry": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                ctypes.c_char_p, ctypes.c_int]),
    "icm_gpu_equity_batched": (ctypes.c_int, [ctypes.c_int, _ip, _ip, _dp, _dp, ctypes.c_int, _dp,
                                              ctypes.POINTER(IcmGpuRunStats)]),
    "icm_gpu_measure_fp64_gflops": (ctypes.c_int, [_dp]),
    "icm_gb300_leaf_factors": (ctypes.c_int, [ctypes.c_int, _dp, _dp]),
    "icm_gpu_last_launch_count": (ctypes.c_long, []),
    "icm_gb300_plan_set_profiling": (ctypes.c_int, [_vp, ctypes.c_int]),
    "icm_gb300_plan_kernel_stats": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_char_p, ctypes.c_int, _dp,
                                                   ctypes.POINTER(ctypes.c_long), _dp]),
    "icm_gb300_plan_device_ms": (ctypes.c_double, [_vp]),
    "icm_gpu_equity_noalloc": (ctypes.c_int, [ctypes.c_int, _dp, ctypes.c_int, _dp, ctypes.c_int, _dp]),
    "icm_gb300_equity_vjp": (ctypes.c_int, [ctypes.c_int, _dp, ctypes.c_int, _dp, ctypes.c_int, _dp, _dp, _dp,
                                            ctypes.c_int]),
    "icm_gb300_vjp_create": (_vp, [ctypes.c_int, _dp, ctypes.c_int]),
    "icm_gb300_vjp_run": (ctypes.c_int, [_vp, ctypes.c_int, _dp, _dp, _dp, _dp, ctypes.c_int,
                                         ctypes.POINTER(IcmGpuRunStats)]),
    "icm_gb300_vjp_destroy": (None, [_vp]),
    "icm_gb300_vjp_device_ms": (ctypes.c_double, [_vp]),
    "icm_gb300_equity_vjp_batched": (ctypes.c_int, [ctypes.c_int, _ip, _ip, _dp, _dp, ctypes.c_int, _dp, _dp, _dp,
                                                    ctypes.c_int]),
    "icm_gb300_tuner_load": (ctypes.c_int, [ctypes.c_char_p]),
    "icm_gb300_tuner_save": (ctypes.c_int, [ctypes.c_char_p]),
    "icm_gb300_tuner_clear": (None, []),
    "icm_gb300_tuner_lookup": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _ip, _ip]),
    "icm_gb300_tuner_lookup_level": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, _ip, _ip]),
    "icm_gb300_autotune": (ctypes.c_int, [ctypes.c_int, _dp, ctypes.c_int, _dp, ctypes.c_int, ctypes.c_int, _ip, _ip,
                                          _dp]),
    "icm_gb300_equity_adaptive": (ctypes.c_int, [ctypes.c_int, _dp, _dp, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                                 ctypes.c_int, _dp, _ip, _dp]),
    "icm_gb300_batch_create": (_vp, [ctypes.c_int, _ip, _ip, _dp]),
    "icm_gb300_vjp_batch_create": (_vp, [ctypes.c_int, _ip, _ip, _dp]),
    "icm_gb300_vjp_batch_run": (ctypes.c_int, [_vp, ctypes.c_int, _dp, _dp, _dp, _dp, ctypes.c_int,
                                               ctypes.POINTER(IcmGpuRunStats)]),
    "icm_gb300_batch_run": (ctypes.c_int, [_vp, ctypes.c_int, _dp, _dp, ctypes.POINTER(IcmGpuRunStats)]),
    "icm_gb300_batch_destroy": (None, [_vp]),
    "icm_gb300_batch_set_options": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int]),
    "icm_gb300_batch_info": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_long), ctypes.POINTER(ctypes.c_long),
                                            ctypes.POINTER(ctypes.c_long), _ip, _dp,
                                            ctypes.POINTER(ctypes.c_size_t)]),
    "icm_gb300_batch_kernel_stats": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_char_p, ctypes.c_int, _dp,
                                                    ctypes.POINTER(ctypes.c_long), _dp]),
}

_lib = None


def library_path() -> str:
    return os.environ.get("ICM_GB300_LIB") or os.path.join(PKG, LIBNAME)


def lib():
    """The loaded library; raises ICMError when it is missing (no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not os.path.isfile(path):
        raise ICMError(f"{path} not found: build it with `python -m icm_gb300.build` "
                       "(the GB300 engine has no CPU fallback)")
    try:
        L = ctypes.CDLL(path)
    except OSError as e:
        raise ICMError(f"Failed to load {path}: {e}") from e
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L
