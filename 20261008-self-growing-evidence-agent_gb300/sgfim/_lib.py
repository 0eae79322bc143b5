"""ctypes binding of libsgfim.so (declarations mirror include/sgfim.h).

The shared library is the product: there is no Python or CPU fallback.
Loading fails with an ImportError-like ``RuntimeError`` when the library has
not been built.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libsgfim.so")

u64p = C.POINTER(C.c_uint64)
u32p = C.POINTER(C.c_uint32)
u16p = C.POINTER(C.c_uint16)
f32p = C.POINTER(C.c_float)
f64p = C.POINTER(C.c_double)

OK, EINVAL, ENOMEM, EIO, EDEVICE, ESTATE, ETIMEDOUT, ECANCELED, ENODATA = 0, -1, -2, -3, -4, -5, -6, -7, -8
ECAPACITY = -9
NOALLOC_MAX_CAND = 1048576
ROOTS_ALL, ROOTS_LIST, ROOTS_MINCOUNT = 0, 1, 2
ORDER_SUPPORT, ORDER_LEARNED, ORDER_SUPPORT_DESC = 0, 1, 2
TRACE_DIM = 8
COOC_AUTO, COOC_POPC, COOC_BMMA, COOC_TC_F8, COOC_TC_F8_256 = 0, 1, 2, 3, 4


class Config(C.Structure):
    _fields_ = [("device", C.c_int), ("hbm_budget", C.c_uint64), ("wave_nodes", C.c_uint32),
                ("flags", C.c_uint32), ("tune_cache", C.c_char_p), ("wait_limit_us", C.c_uint32)]


class DatasetInfo(C.Structure):
    _fields_ = [("n_txn", C.c_uint64), ("n_ids", C.c_uint32), ("n_present", C.c_uint32),
                ("id_min", C.c_uint32), ("id_max", C.c_uint32), ("len_min", C.c_uint64),
                ("len_max", C.c_uint64), ("len_mean", C.c_double), ("words", C.c_uint64),
                ("rows", C.c_uint32)]


class Result(C.Structure):
    _fields_ = [("n_sets", C.c_uint64), ("set_ptr", u64p), ("items", u32p), ("support", u32p),
                ("emit_time_s", f64p), ("n_txn", C.c_uint64), ("min_count", C.c_uint32),
                ("elapsed_s", C.c_double), ("preprocess_s", C.c_double), ("nodes", C.c_uint64),
                ("waves", C.c_uint64), ("kernel_launches", C.c_uint64), ("candidates", C.c_uint64),
                ("trace_n", C.c_uint64), ("trace_dim", C.c_uint32), ("trace_features", f32p),
                ("trace_labels", C.POINTER(C.c_uint8)), ("phase_s", C.c_double * 8), ("emit_node", u64p)]


class MineParams(C.Structure):
    _fields_ = [("min_count", C.c_uint32), ("root_rule", C.c_uint32), ("roots", u32p),
                ("n_roots", C.c_uint32), ("root_min_count", C.c_uint32), ("order", C.c_uint32),
                ("time_limit_s", C.c_double), ("node_limit", C.c_uint64), ("record_trace", C.c_uint32)]


class Checkpoint(C.Structure):
    _fields_ = [("t_s", C.c_double), ("elapsed_s", C.c_double), ("n_emitted", C.c_uint64),
                ("set_ptr", u64p), ("items", u32p), ("support", u32p), ("nodes", C.c_uint64)]


CKPT_CB = C.CFUNCTYPE(C.c_int, C.c_void_p, C.POINTER(Checkpoint))


class PhaseStats(C.Structure):
    _fields_ = [("calls", C.c_uint64), ("launches", C.c_uint64), ("prep_ms", C.c_double),
                ("count_ms", C.c_double), ("tail_ms", C.c_double)]


F_VERBOSE, F_IGNORE_ID0, F_PHASE_TIMERS, F_BLOCKING_SYNC = 0x1, 0x2, 0x4, 0x8
F_WINDOWS_HORIZONTAL = 0x10
F_NO_PROJECTION, F_PROJECT = 0x20, 0x40
TX_LOAD = 0x1
TX_P2_FULL = 0x2


class WindowsResult(C.Structure):
    _fields_ = [("n_windows", C.c_uint64), ("mask_words", C.c_uint32), ("offset", u64p), ("masks", u64p),
                ("support", u32p), ("status", C.POINTER(C.c_int32)), ("nodes", u64p),
                ("batched", C.POINTER(C.c_uint8)), ("elapsed_s", C.c_double), ("kernel_ms", C.c_double),
                ("launches", C.c_uint32), ("warps", C.c_uint32), ("tasks", C.c_uint64),
                ("task_kernel_ms", C.c_double), ("task_ms_max", C.c_double), ("task_ms_sum", C.c_double)]


class TfMeta(C.Structure):
    _fields_ = [("trans_set_file", C.c_char_p), ("support_threshold", C.c_double),
                ("computation_time_s", C.c_double), ("preprocessing_time_s", C.c_double),
                ("dimension_reduced", C.c_uint32)]


class AfMeta(C.Structure):
    _fields_ = [("trans_set_file", C.c_char_p), ("upto_stage", C.c_uint32),
                ("preprocessing_time_s", C.c_double), ("runtime_per_stage_s", f64p),
                ("frequency_thr_per_stage", u32p)]


# name -> (restype, argtypes); every symbol include/sgfim.h declares
SIGNATURES = {
    "sgfim_abi_version": (C.c_int, []),
    "sgfim_open": (C.c_int, [C.POINTER(Config), C.POINTER(C.c_void_p)]),
    "sgfim_close": (None, [C.c_void_p]),
    "sgfim_last_error": (C.c_char_p, [C.c_void_p]),
    "sgfim_device_status": (C.c_int, [C.c_void_p, C.c_void_p]),
    "sgfim_selftest_wait": (C.c_int, [C.c_void_p]),
    "sgfim_noalloc_status": (C.c_int, [C.c_void_p]),
    "sgfim_load_fimi": (C.c_int, [C.c_void_p, C.c_char_p]),
    "sgfim_load_csr": (C.c_int, [C.c_void_p, u64p, u32p, C.c_uint64]),
    "sgfim_load_bitmaps": (C.c_int, [C.c_void_p, u64p, C.c_uint32, C.c_uint64, C.c_uint64]),
    "sgfim_dataset_info_get": (C.c_int, [C.c_void_p, C.POINTER(DatasetInfo)]),
    "sgfim_item_counts": (C.c_int, [C.c_void_p, u32p, C.c_uint32]),
    "sgfim_support_batch": (C.c_int, [C.c_void_p, u64p, u32p, C.c_uint64, u32p]),
    "sgfim_support_batch_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint64, C.c_uint64,
                                             C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p]),
    "sgfim_phase_stats_get": (C.c_int, [C.c_void_p, C.POINTER(PhaseStats), C.c_int]),
    "sgfim_support_plan_set": (C.c_int, [C.c_void_p, C.c_int, C.c_uint32, C.c_uint32]),
    "sgfim_ring_open": (C.c_int, [C.c_int, C.c_uint32, C.c_uint64, C.POINTER(C.c_void_p)]),
    "sgfim_ring_close": (None, [C.c_void_p]),
    "sgfim_ring_head": (C.c_uint64, [C.c_void_p]),
    "sgfim_ring_capacity": (C.c_uint64, [C.c_void_p]),
    "sgfim_ring_append": (C.c_int, [C.c_void_p, u64p, u32p, C.c_uint64]),
    "sgfim_ring_window_load": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_uint64]),
    "sgfim_ring_mine_windows": (C.c_int, [C.c_void_p, C.c_void_p, u64p, u64p, u32p, C.c_uint64,
                                          C.POINTER(C.POINTER(WindowsResult))]),
    "sgfim_windows_result_free": (None, [C.POINTER(WindowsResult)]),
    "sgfim_transactionize": (C.c_int, [C.c_void_p, f64p, C.c_uint64, C.c_uint32, C.POINTER(C.c_int32), C.c_uint32,
                                       C.c_uint32, C.c_uint32, C.c_uint32, f64p, u32p, u32p, C.POINTER(C.c_int32),
                                       u64p]),
    "sgfim_transactionize_online": (C.c_int, [C.c_void_p, f64p, C.c_uint64, C.c_uint32, C.POINTER(C.c_int32),
                                              C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, f64p, u32p,
                                              C.POINTER(C.c_int32), u64p]),
    "sgfim_support_batch_noalloc": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint64, C.c_uint64, C.c_void_p,
                                              C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p]),
    "sgfim_cooccurrence": (C.c_int, [C.c_void_p, u32p, C.c_uint32]),
    "sgfim_cooccurrence_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint64, C.c_uint64,
                                            C.c_void_p, C.c_int, C.c_void_p]),
    "sgfim_frequent_extensions": (C.c_int, [C.c_void_p, u64p, u32p, C.c_uint64, C.c_uint32, u64p, C.c_uint32]),
    "sgfim_mine": (C.c_int, [C.c_void_p, C.POINTER(MineParams), C.POINTER(C.POINTER(Result))]),
    "sgfim_mine_anytime": (C.c_int, [C.c_void_p, C.POINTER(MineParams), f64p, C.c_uint32, CKPT_CB,
                                     C.c_void_p, C.POINTER(C.POINTER(Result))]),
    "sgfim_result_free": (None, [C.POINTER(Result)]),
    "sgfim_write_tensorfim": (C.c_int, [C.c_void_p, C.POINTER(Result), C.POINTER(TfMeta), C.c_char_p]),
    "sgfim_write_anyfim": (C.c_int, [C.c_void_p, C.POINTER(C.POINTER(Result)), C.POINTER(AfMeta), C.c_char_p]),
    "sgfim_load_scorer": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, u16p, f32p, u16p, f32p, u16p, f32p]),
    "sgfim_mlp_forward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32] +
                          [C.c_void_p] * 9 + [C.c_void_p]),
    "sgfim_mlp_backward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32] +
                           [C.c_void_p] * 7 + [C.c_float] + [C.c_void_p] * 7 + [C.c_void_p]),
    "sgfim_adam_step": (C.c_int, [C.c_void_p] * 6 + [C.c_uint32, C.c_float, C.c_float, C.c_float, C.c_float,
                                                     C.c_uint32, C.c_float, C.c_void_p]),
}

_lib = None


def load(path=None):
    """Load libsgfim.so once; raises RuntimeError when it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError(f"libsgfim.so not built at {path}; run __graft_entry__.build() "
                           "or python -m sgfim.build")
    L = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L
