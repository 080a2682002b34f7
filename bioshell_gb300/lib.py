"""ctypes binding of ``libbioshell_crmsd.so`` (declarations in
``include/bioshell_crmsd.h``).

The library is loaded from the package's ``lib/`` directory.  There is no
fallback: if the shared library is missing or cannot be loaded, importing the
binding raises, and every compute call needs a usable sm_103 GPU.
"""
from __future__ import annotations

import ctypes
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libbioshell_crmsd.so")

BS_OK = 0
STATUS_NAMES = {
    0: "BS_OK", 1: "BS_ERR_INVALID_ARG", 2: "BS_ERR_CUDA", 3: "BS_ERR_OOM", 4: "BS_ERR_TIMEOUT",
    5: "BS_ERR_UNSUPPORTED", 6: "BS_ERR_NONFINITE", 7: "BS_ERR_BUDGET", 8: "BS_ERR_NO_DEVICE",
    9: "BS_ERR_INTERNAL", 10: "BS_ERR_CANCELLED",
}
PRECISION = {"plain64": 0, "mixed": 1}
LAYOUT = {"triangle": 0, "square": 1}
OUT_TYPE = {"f64": 0, "f32": 1}
LINK = {"single": 0, "complete": 1, "average": 2, "median": 3, "centroid": 4, "ward": 5}
FLAG_NO_GRAPH = 1
FLAG_AUTOTUNE = 2


class bs_opts(ctypes.Structure):
    _fields_ = [("version", ctypes.c_uint32), ("precision", ctypes.c_int32), ("layout", ctypes.c_int32),
                ("out_type", ctypes.c_int32), ("tolerance", ctypes.c_double), ("flags", ctypes.c_int32),
                ("flag_queue", ctypes.c_int32), ("row_begin", ctypes.c_int32), ("row_end", ctypes.c_int32),
                ("reserved", ctypes.c_int32 * 4)]


class bs_set_desc(ctypes.Structure):
    _fields_ = [("xyz", ctypes.c_void_p), ("n", ctypes.c_int64), ("L", ctypes.c_int32),
                ("reserved", ctypes.c_int32), ("out", ctypes.c_void_p)]


class bs_metrics(ctypes.Structure):
    _fields_ = [("pairs", ctypes.c_int64), ("pairs_refined", ctypes.c_int64), ("ms_total", ctypes.c_double),
                ("ms_h2d", ctypes.c_double), ("ms_prep", ctypes.c_double), ("ms_main", ctypes.c_double),
                ("ms_refine", ctypes.c_double), ("ms_d2h", ctypes.c_double), ("scale_exp", ctypes.c_int32),
                ("main_launches", ctypes.c_int32), ("jobs", ctypes.c_int32), ("graph", ctypes.c_int32),
                ("quant_bound", ctypes.c_double),
                ("bytes_h2d", ctypes.c_int64), ("bytes_d2h", ctypes.c_int64), ("narrow_jobs", ctypes.c_int32),
                ("tuned_classes", ctypes.c_int32), ("pairs_plain", ctypes.c_int64)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class bs_server_config(ctypes.Structure):
    _fields_ = [("nbuckets", ctypes.c_int32), ("bucket_L", ctypes.POINTER(ctypes.c_int32)),
                ("bucket_n", ctypes.POINTER(ctypes.c_int64)), ("bucket_xyz", ctypes.POINTER(ctypes.c_void_p)),
                ("top_k", ctypes.c_int32), ("max_inflight", ctypes.c_int32), ("hbm_budget", ctypes.c_size_t),
                ("precision", ctypes.c_int32), ("max_batch_rows", ctypes.c_int32), ("tolerance", ctypes.c_double),
                ("index_min", ctypes.c_int32), ("reserved", ctypes.c_int32 * 5)]


class bs_server_stats(ctypes.Structure):
    _fields_ = [("queries_done", ctypes.c_int64), ("clusters_done", ctypes.c_int64), ("pairs", ctypes.c_int64),
                ("batches", ctypes.c_int64), ("plain_fallbacks", ctypes.c_int64), ("pending", ctypes.c_int64),
                ("p50_ms", ctypes.c_double), ("p99_ms", ctypes.c_double), ("max_ms", ctypes.c_double),
                ("mean_ms", ctypes.c_double), ("cluster_p50_ms", ctypes.c_double),
                ("cluster_p99_ms", ctypes.c_double), ("pairs_per_s", ctypes.c_double),
                ("mean_batch_rows", ctypes.c_double), ("seconds", ctypes.c_double),
                ("pairs_screened", ctypes.c_int64)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


_dp = ctypes.POINTER(ctypes.c_double)
_fp = ctypes.POINTER(ctypes.c_float)
_i64p = ctypes.POINTER(ctypes.c_int64)
_i32p = ctypes.POINTER(ctypes.c_int32)
_vp = ctypes.c_void_p

# (name, restype, argtypes) for every function the header declares
SIGNATURES = [
    ("bs_abi_version", ctypes.c_int32, []),
    ("bs_status_string", ctypes.c_char_p, [ctypes.c_int32]),
    ("bs_last_error", ctypes.c_char_p, [_vp]),
    ("bs_ctx_create", ctypes.c_int32, [ctypes.POINTER(_vp), ctypes.c_int32, ctypes.c_size_t]),
    ("bs_ctx_destroy", None, [_vp]),
    ("bs_opts_init", None, [ctypes.POINTER(bs_opts)]),
    ("bs_get_metrics", ctypes.c_int32, [_vp, ctypes.POINTER(bs_metrics)]),
    ("bs_ctx_trim", ctypes.c_int32, [_vp]),
    ("bs_ctx_stream", ctypes.c_void_p, [_vp]),
    ("bs_crmsd", ctypes.c_int32, [_vp, _vp, _vp, ctypes.c_int32, _dp]),
    ("bs_superpose", ctypes.c_int32, [_vp, _vp, _vp, ctypes.c_int32, _vp, _vp, _vp]),
    ("bs_superpose_pairs", ctypes.c_int32, [_vp, _vp, ctypes.c_int64, ctypes.c_int32, _vp, _vp, ctypes.c_int64, _vp,
                                            _vp, _vp]),
    ("bs_all_vs_all", ctypes.c_int32, [_vp, _vp, ctypes.c_int64, ctypes.c_int32, ctypes.POINTER(bs_opts), _vp]),
    ("bs_tune_get", ctypes.c_int32, [_vp, ctypes.c_int32, ctypes.c_int64, _i32p]),
    ("bs_tune_set", ctypes.c_int32, [_vp, ctypes.c_int32, ctypes.c_int64, ctypes.c_int32]),
    ("bs_batched", ctypes.c_int32, [_vp, ctypes.POINTER(bs_set_desc), ctypes.c_int32, ctypes.POINTER(bs_opts)]),
    ("bs_pairs", ctypes.c_int32, [_vp, _vp, ctypes.c_int64, ctypes.c_int32, _vp, _vp, ctypes.c_int64,
                                  ctypes.POINTER(bs_opts), _vp]),
    ("bs_all_vs_all_static", ctypes.c_int32, [_vp, ctypes.c_int64, ctypes.c_int32, _vp, _vp]),
    ("bs_server_create", ctypes.c_int32, [ctypes.POINTER(_vp), ctypes.c_int32, ctypes.POINTER(bs_server_config)]),
    ("bs_server_destroy", None, [_vp]),
    ("bs_server_last_error", ctypes.c_char_p, [_vp]),
    ("bs_server_submit", ctypes.c_int32, [_vp, _vp, ctypes.c_int32, ctypes.c_int32, _i64p]),
    ("bs_server_submit_cluster", ctypes.c_int32, [_vp, _vp, ctypes.c_int64, ctypes.c_int32, ctypes.c_double,
                                                  ctypes.c_int32, _i64p]),
    ("bs_server_poll", ctypes.c_int32, [_vp, ctypes.c_int64, _i32p]),
    ("bs_server_wait", ctypes.c_int32, [_vp, ctypes.c_int64, _vp, _vp, ctypes.c_double]),
    ("bs_server_wait_cluster", ctypes.c_int32, [_vp, ctypes.c_int64, _vp, ctypes.c_double]),
    ("bs_server_get_stats", ctypes.c_int32, [_vp, ctypes.POINTER(bs_server_stats)]),
    ("bs_server_cancel", ctypes.c_int32, [_vp, ctypes.c_int64, ctypes.POINTER(ctypes.c_int32)]),
    ("bs_server_reset_stats", ctypes.c_int32, [_vp]),
    ("bs_hierarchical", ctypes.c_int32, [_vp, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32, _i64p, _fp]),
    ("bs_cut_tree", ctypes.c_int32, [_i64p, _fp, ctypes.c_int64, ctypes.c_float, _i64p]),
    ("bs_optics", ctypes.c_int32, [_vp, ctypes.c_int64, ctypes.c_int32, ctypes.c_double, ctypes.c_int32, _i64p,
                                   _dp, _i64p]),
    ("bs_neighbors", ctypes.c_int32, [_vp, _vp, ctypes.c_int64, ctypes.c_int32, ctypes.c_double,
                                      ctypes.POINTER(bs_opts), _i64p]),
    ("bs_neighbors_get", ctypes.c_int32, [_vp, _vp, _vp, _vp]),
    ("bs_hierarchical_gpu", ctypes.c_int32, [_vp, _vp, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32, _i64p, _fp]),
    ("bs_optics_neighbors", ctypes.c_int32, [_i64p, _i32p, _fp, ctypes.c_int64, ctypes.c_double, ctypes.c_int32,
                                             _i64p, _dp, _i64p]),
    ("bs_io_last_error", ctypes.c_char_p, []),
    ("bs_models_read", ctypes.c_int32, [ctypes.c_char_p, ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(_vp), _i64p,
                                        _i32p]),
    ("bs_models_copy", ctypes.c_int32, [_vp, _vp]),
    ("bs_models_free", None, [_vp]),
    ("bs_tsv_write", ctypes.c_int32, [ctypes.c_char_p, _vp, ctypes.c_int64, ctypes.c_int32, _vp, ctypes.c_int32]),
    ("bs_tsv_read", ctypes.c_int32, [ctypes.c_char_p, ctypes.c_double, ctypes.c_int32, ctypes.POINTER(_vp), _i64p]),
    ("bs_tsv_matrix", ctypes.c_int32, [_vp, _fp]),
    ("bs_tsv_label", ctypes.c_char_p, [_vp, ctypes.c_int64]),
    ("bs_tsv_free", None, [_vp]),
    ("bs_host_alloc", ctypes.c_int32, [ctypes.c_size_t, ctypes.POINTER(_vp)]),
    ("bs_host_free", ctypes.c_int32, [_vp]),
    ("bs_selftest_digits", ctypes.c_int32, [_dp, ctypes.c_int32, ctypes.c_int32, _i32p, _i64p, _dp]),
    ("bs_selftest_epilogue", ctypes.c_int32, [_fp, ctypes.c_int64, ctypes.c_int64, ctypes.c_double, ctypes.c_double,
                                              ctypes.c_double, ctypes.c_int32, ctypes.c_int32, ctypes.c_double, _dp,
                                              _i32p]),
    ("bs_selftest_exact", ctypes.c_int32, [_i32p, _i32p, ctypes.c_int32, ctypes.c_int32, _dp]),
    ("bs_selftest_superpose", ctypes.c_int32, [_vp, _vp, ctypes.c_int32, _vp, _vp, _vp]),
    ("bs_selftest_bands", ctypes.c_int32, [ctypes.c_int64, ctypes.c_int32, _vp, ctypes.c_int32, _vp]),
    ("bs_selftest_screen", ctypes.c_int32, [_fp, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int32,
                                            ctypes.c_int32, _fp, _fp]),
    ("bs_debug_tile_levels", ctypes.c_int32, [_vp, _vp, ctypes.c_int64, ctypes.c_int32, _fp]),
    ("bs_debug_set_wait_limit", ctypes.c_int32, [_vp, ctypes.c_int64]),
    ("bs_partition_rows", ctypes.c_int32, [ctypes.c_int64, ctypes.c_int32, _vp]),
    ("bs_tune_list", ctypes.c_int32, [_vp, _vp, _vp, _vp, ctypes.c_int32, _vp, _vp]),
    ("bs_debug_fail_alloc", ctypes.c_int32, [_vp, ctypes.c_int64]),
    ("bs_debug_pair_levels", ctypes.c_int32, [_vp, _vp, ctypes.c_int64, ctypes.c_int32, _vp, _vp, ctypes.c_int64,
                                              _fp, _dp]),
    ("bs_diag_fp64_peak", ctypes.c_int32, [ctypes.c_int32, _dp]),
]

_lib = None
_lock = threading.Lock()


def load():
    """Load the engine library (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with `python -m bioshell_gb300._build` "
                              "(the engine has no CPU fallback)")
        lib = ctypes.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


class CrmsdError(RuntimeError):
    """A non-zero bs_status from the engine."""

    def __init__(self, status: int, message: str):
        self.status = status
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
