"""ctypes binding of libdynlp_gb300.so (include/dlp_gb300.h).

The library is the product: this module only declares its C ABI. Loading
fails loudly when the shared library has not been built; there is no Python
or CPU fallback for any compute entry point.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = Path(os.environ.get("DLP_LIBRARY", PKG / "_build" / "libdynlp_gb300.so"))

c_int_p = ctypes.POINTER(ctypes.c_int)
c_float_p = ctypes.POINTER(ctypes.c_float)
c_void_p = ctypes.c_void_p


class BatchView(ctypes.Structure):
    _fields_ = [
        ("inserted", c_void_p), ("num_inserted", ctypes.c_int),
        ("gt_ids", c_void_p), ("gt_labels", c_void_p), ("num_gt", ctypes.c_int),
        ("deleted", c_void_p), ("num_deleted", ctypes.c_int),
        ("edge_src", c_void_p), ("edge_dst", c_void_p), ("edge_weight", c_void_p),
        ("num_edges", ctypes.c_int),
    ]


class Config(ctypes.Structure):
    _fields_ = [
        ("tau", ctypes.c_float), ("delta", ctypes.c_float), ("max_iterations", ctypes.c_int),
        ("semantics", ctypes.c_int), ("device", ctypes.c_int), ("record", ctypes.c_int),
        ("narrow_lanes", ctypes.c_int), ("blocks_per_sm", ctypes.c_int),
        ("wait_timeout_s", ctypes.c_double), ("small_frontier_solo", ctypes.c_int),
        ("solo_entry", ctypes.c_int), ("subgrid_entry", ctypes.c_int), ("arithmetic", ctypes.c_int),
    ]


class BatchStats(ctypes.Structure):
    _fields_ = [
        ("batch", ctypes.c_int), ("iterations", ctypes.c_int), ("num_components", ctypes.c_int),
        ("num_sub_edges", ctypes.c_int), ("hook_edges", ctypes.c_int), ("hook_rounds", ctypes.c_int),
        ("seed_frontier", ctypes.c_int), ("seed_marks", ctypes.c_int),
        ("affected_edges", ctypes.c_int64), ("frontier_visits", ctypes.c_int64),
        ("correct", ctypes.c_int64), ("total", ctypes.c_int64), ("accuracy", ctypes.c_float),
        ("status", ctypes.c_int), ("init_branch", ctypes.c_int), ("hook_truncated", ctypes.c_int),
        ("device_ms", ctypes.c_float), ("dirty_rows", ctypes.c_int), ("dirty_entries", ctypes.c_int64),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class ServerConfig(ctypes.Structure):
    _fields_ = [
        ("slice_us", ctypes.c_double), ("pass_budget", ctypes.c_int),
        ("memory_budget_bytes", ctypes.c_size_t), ("max_batches_per_step", ctypes.c_int),
        ("serial", ctypes.c_int), ("evict_idle", ctypes.c_int),
    ]


class Request(ctypes.Structure):
    _fields_ = [
        ("graph_id", ctypes.c_int), ("batch_index", ctypes.c_int), ("batch", BatchView),
        ("arrival_s", ctypes.c_double),
    ]


class RequestResult(ctypes.Structure):
    _fields_ = [
        ("graph_id", ctypes.c_int), ("batch_index", ctypes.c_int), ("status", ctypes.c_int),
        ("arrival_s", ctypes.c_double), ("admit_s", ctypes.c_double), ("finish_s", ctypes.c_double),
        ("steps", ctypes.c_int), ("stats", BatchStats),
    ]


class TuneReport(ctypes.Structure):
    _fields_ = [
        ("candidates", ctypes.c_int), ("best", ctypes.c_int), ("lanes", ctypes.c_int * 32),
        ("blocks_per_sm", ctypes.c_int * 32), ("solo_entry", ctypes.c_int * 32),
        ("subgrid_entry", ctypes.c_int * 32), ("ms", ctypes.c_double * 32),
    ]


# enum dlp_arithmetic
ARITH_IEEE, ARITH_REFERENCE_FAST_MATH = 0, 1

# status codes
DLP_OK = 0
DLP_ERR_INVALID_ARGUMENT = 1
DLP_ERR_CUDA = 2
DLP_ERR_OUT_OF_MEMORY = 3
DLP_ERR_TIMEOUT = 4
DLP_ERR_NO_DEVICE = 5
DLP_ERR_NOT_CONVERGED = 6
DLP_ERR_INTERNAL = 7

SEMANTICS_REF = 0
SEMANTICS_SPEC = 1

ART_SEED_MARKS = 0
ART_FRONTIER0 = 1
ART_SUB_EDGES = 2
ART_COMP_ROOT = 3
ART_INIT_LABELS = 5
ART_FRONTIER_SIZES = 6
ART_ROW_LENGTHS = 7
ART_LABELS = 10

# name -> (restype, argtypes); the declaration list mirrors include/dlp_gb300.h
_I = ctypes.c_int
_P = c_void_p
_SIGNATURES = {
    "dlp_abi_version": (_I, []),
    "dlp_status_string": (ctypes.c_char_p, [_I]),
    "dlp_last_error": (ctypes.c_char_p, []),
    "dlp_problem_generate": (_I, [_I, _I, _I, ctypes.c_uint, ctypes.c_float, ctypes.c_float, ctypes.POINTER(_P)]),
    "dlp_problem_free": (None, [_P]),
    "dlp_problem_num_nodes": (_I, [_P]),
    "dlp_problem_num_edges": (ctypes.c_int64, [_P]),
    "dlp_problem_num_batches": (_I, [_P]),
    "dlp_problem_row_ptr": (_P, [_P]),
    "dlp_problem_col_ind": (_P, [_P]),
    "dlp_problem_values": (_P, [_P]),
    "dlp_problem_true_labels": (_P, [_P]),
    "dlp_problem_batch": (_I, [_P, _I, ctypes.POINTER(BatchView)]),
    "dlp_problem_write_csr": (_I, [_P, ctypes.c_char_p]),
    "dlp_problem_save": (_I, [_P, ctypes.c_char_p]),
    "dlp_problem_load": (_I, [ctypes.c_char_p, ctypes.POINTER(_P)]),
    "dlp_problem_generate_cached": (_I, [_I, _I, _I, ctypes.c_uint, ctypes.c_float, ctypes.c_float, ctypes.c_char_p,
                                         ctypes.POINTER(_P), ctypes.POINTER(_I)]),
    "dlp_mean_edge_weight": (ctypes.c_float, [ctypes.c_int64, _P, _P]),
    "dlp_config_default": (None, [ctypes.POINTER(Config)]),
    "dlp_session_create": (_I, [ctypes.POINTER(Config), _I, ctypes.c_int64, _P, _P, _P, _P, _P, ctypes.POINTER(_P)]),
    "dlp_session_destroy": (_I, [_P]),
    "dlp_session_reset": (_I, [_P]),
    "dlp_session_tau": (ctypes.c_float, [_P]),
    "dlp_session_apply_batch": (_I, [_P, _I, ctypes.POINTER(BatchView), ctypes.POINTER(BatchStats)]),
    "dlp_session_apply_batch_device": (_I, [_P, _I, ctypes.POINTER(BatchView)]),
    "dlp_session_synchronize": (_I, [_P]),
    "dlp_session_stats": (_I, [_P, _I, ctypes.POINTER(BatchStats)]),
    "dlp_session_read_labels": (_I, [_P, _P]),
    "dlp_session_stream": (_P, [_P]),
    "dlp_session_elapsed_ms": (_I, [_P, _I, _I, ctypes.POINTER(ctypes.c_float)]),
    "dlp_irlp": (_I, [_P, _P, _P, _P, _P, _P, _I, ctypes.c_float, _I, c_int_p, _P]),
    "dlp_session_artefact": (_I, [_P, _I, _P, ctypes.c_int64, ctypes.POINTER(ctypes.c_int64)]),
    "dlp_engine_create": (_I, [ctypes.POINTER(Config), _I, ctypes.c_size_t, ctypes.POINTER(_P)]),
    "dlp_engine_destroy": (_I, [_P]),
    "dlp_engine_graph_bytes": (ctypes.c_size_t, [_I, ctypes.c_int64, _I, _I, _I]),
    "dlp_engine_bytes_in_use": (ctypes.c_size_t, [_P]),
    "dlp_engine_add_graph": (_I, [_P, _I, ctypes.c_int64, _P, _P, _P, _P, _P, c_int_p]),
    "dlp_engine_remove_graph": (_I, [_P, _I]),
    "dlp_engine_reset_graph": (_I, [_P, _I]),
    "dlp_engine_tau": (ctypes.c_float, [_P, _I]),
    "dlp_engine_stream": (_P, [_P]),
    "dlp_engine_step": (_I, [_P, _I, _P, _P, ctypes.POINTER(BatchView), ctypes.POINTER(BatchStats)]),
    "dlp_engine_step_device": (_I, [_P, _I, _P, _P, ctypes.POINTER(BatchView)]),
    "dlp_engine_synchronize": (_I, [_P]),
    "dlp_engine_stats": (_I, [_P, _I, _I, ctypes.POINTER(BatchStats)]),
    "dlp_engine_steps": (_I, [_P]),
    "dlp_engine_debug": (_I, [_P, c_int_p]),
    "dlp_session_debug": (_I, [_P, c_int_p]),
    "dlp_engine_elapsed_ms": (_I, [_P, _I, _I, ctypes.POINTER(ctypes.c_float)]),
    "dlp_engine_read_labels": (_I, [_P, _I, _P]),
    "dlp_engine_artefact": (_I, [_P, _I, _I, _P, ctypes.c_int64, ctypes.POINTER(ctypes.c_int64)]),
    "dlp_engine_step_sliced": (_I, [_P, _I, _P, _P, ctypes.POINTER(BatchView), _I, ctypes.c_double, c_int_p, c_int_p,
                                    c_int_p]),
    "dlp_engine_graph_nodes": (_I, [_P, _I]),
    "dlp_engine_snapshot": (_I, [_P, _I, _P, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]),
    "dlp_engine_restore": (_I, [_P, _P, ctypes.c_size_t, c_int_p]),
    "dlp_engine_restore_as": (_I, [_P, _P, ctypes.c_size_t, _I]),
    "dlp_engine_graph_resident_bytes": (ctypes.c_size_t, [_P, _I]),
    "dlp_engine_hold_id": (_I, [_P, _I]),
    "dlp_engine_pass_modes": (_I, [_P, _P, _P]),
    "dlp_session_pass_modes": (_I, [_P, _P, _P]),
    "dlp_engine_release_id": (_I, [_P, _I]),
    "dlp_server_evictions": (_I, [_P, c_int_p, c_int_p]),
    "dlp_server_make_resident": (_I, [_P, _I]),
    "dlp_autotune": (_I, [ctypes.POINTER(Config), _I, c_int_p, c_int_p, _I, _I, ctypes.POINTER(TuneReport)]),
    "dlp_engine_reserve": (_I, [_P, _I, _I, _I]),
    "dlp_server_reserve": (_I, [_P, _I, _I, _I, _I, _I]),
    "dlp_engine_in_progress": (_I, [_P, _I]),
    "dlp_server_config_default": (None, [ctypes.POINTER(ServerConfig)]),
    "dlp_server_create": (_I, [_P, ctypes.POINTER(ServerConfig), ctypes.POINTER(_P)]),
    "dlp_server_destroy": (_I, [_P]),
    "dlp_server_clock": (ctypes.c_double, [_P]),
    "dlp_server_submit": (_I, [_P, ctypes.POINTER(Request), c_int_p]),
    "dlp_server_poll": (_I, [_P, c_int_p, _I, c_int_p]),
    "dlp_server_result": (_I, [_P, _I, ctypes.POINTER(RequestResult)]),
    "dlp_server_pending": (_I, [_P]),
    "dlp_server_replay": (_I, [_P, _I, ctypes.POINTER(Request), ctypes.POINTER(RequestResult),
                               ctypes.POINTER(ctypes.c_double)]),
    "dlp_mark_deletions": (_I, [_P, _P, _P, _P, _P, _I, _I, _P]),
    "dlp_build_sparsified_subgraph": (_I, [_P, _P, _P, _P, _P, _P, _P, _P, _I, _P, _I, _P, ctypes.c_float,
                                           _P, _P, _P, c_int_p, c_int_p, _P]),
    "dlp_connected_components": (_I, [_P, _P, _I, _P, _I, _P, c_int_p, _I, _P]),
    "dlp_label_initialization": (_I, [_P, _P, _P, _P, _P, _P, _I, _P, _I, _P, _I, _P]),
    "dlp_iterative_propagation": (_I, [_P, _P, _P, _P, _P, _P, _P, _P, _I, ctypes.c_float, _I, c_int_p, _P]),
    "dlp_iterative_propagation_noalloc": (_I, [_P, _P, _P, _P, _P, _P, _P, _P, _I, ctypes.c_float, _I, c_int_p,
                                               _P]),
    "dlp_device_count": (_I, [c_int_p]),
    "dlp_device_name": (_I, [_I, ctypes.c_char_p, _I]),
    "dlp_set_launcher_arithmetic": (_I, [_I]),
    "dlp_set_device": (_I, [_I]),
    "dlp_malloc": (_I, [ctypes.POINTER(_P), ctypes.c_size_t]),
    "dlp_free": (_I, [_P]),
    "dlp_memcpy_htod": (_I, [_P, _P, ctypes.c_size_t]),
    "dlp_memcpy_dtoh": (_I, [_P, _P, ctypes.c_size_t]),
    "dlp_memset": (_I, [_P, _I, ctypes.c_size_t]),
    "dlp_device_synchronize": (_I, []),
}

_lib = None


class DlpError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{status_name(status)}: {message}")
        self.status = status


def status_name(status: int) -> str:
    names = {0: "DLP_OK", 1: "DLP_ERR_INVALID_ARGUMENT", 2: "DLP_ERR_CUDA", 3: "DLP_ERR_OUT_OF_MEMORY",
             4: "DLP_ERR_TIMEOUT", 5: "DLP_ERR_NO_DEVICE", 6: "DLP_ERR_NOT_CONVERGED", 7: "DLP_ERR_INTERNAL"}
    return names.get(status, f"status {status}")


def lib() -> ctypes.CDLL:
    """Loads the library (once). Raises ImportError when it was not built."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} is missing: build it with `python -m labelpropcuda_gb300.build` "
                          "(there is no CPU fallback)")
    handle = ctypes.CDLL(str(LIB_PATH))
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(handle, name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args
    _lib = handle
    return _lib


def check(status: int) -> None:
    if status != DLP_OK:
        msg = lib().dlp_last_error()
        raise DlpError(status, msg.decode() if msg else "")


def exported_symbols() -> list[str]:
    return list(_SIGNATURES)
