"""ctypes bindings of libsegtaco.so (include/segtaco.h, include/segtaco_taco.h).

The library is the product: every compute call below goes through its C ABI.
There is no fallback -- if the shared library is missing or no CUDA device is
present, the calls raise.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libsegtaco.so")

OK = 0
EINVAL = -1
ECUDA = -2
ENOMEM = -3
ETIMEOUT = -4
EUNSUPPORTED = -5
ECANCELLED = -6
EBUSY = -7

AUTO = -1
RB_SR = 0
RB_PR = 1
EB_SR = 2
EB_PR = 3
SCHEDULES = {"rb_sr": RB_SR, "rb_pr": RB_PR, "eb_sr": EB_SR, "eb_pr": EB_PR}

F32 = 0
BF16 = 1

FLAG_L2_HINTS = 1
FLAG_PARTITION_READY = 2
FLAG_SMEM_RING = 4
FLAG_TMA_BULK = 8
FLAG_ROW_WALK = 16
FLAG_FLAT_WALK = 32
FLAG_LONG_ROWS = 64
FLAG_WINDOW = 128
FLAG_SLOT_WALK = 256


class SegtacoError(RuntimeError):
    def __init__(self, code, message):
        super().__init__("segtaco error %d: %s" % (code, message))
        self.code = code


class Config(C.Structure):
    """segtaco_config: zero fields mean automatic."""
    _fields_ = [("schedule", C.c_int32), ("col_tile", C.c_int32), ("vec", C.c_int32),
                ("rows_per_unit", C.c_int32), ("items_per_unit", C.c_int32),
                ("flags", C.c_uint32), ("depth", C.c_int32), ("k_parts", C.c_int32)]

    @classmethod
    def make(cls, schedule=AUTO, col_tile=0, vec=0, rows_per_unit=0, items_per_unit=0,
             flags=0, depth=0, k_parts=0):
        if isinstance(schedule, str):
            schedule = SCHEDULES[schedule]
        return cls(schedule, col_tile, vec, rows_per_unit, items_per_unit, flags, depth, k_parts)

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class SddmmConfig(C.Structure):
    """segtaco_sddmm_config: kernel, nonzeros per warp block, lanes per dot product."""
    _fields_ = [("kernel", C.c_int32), ("block_nnz", C.c_int32), ("lanes", C.c_int32),
                ("reserved", C.c_int32)]

    @classmethod
    def make(cls, kernel=0, block_nnz=0, lanes=0):
        return cls(kernel, block_nnz, lanes, 0)

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


SDDMM_AUTO, SDDMM_FIXED, SDDMM_GENERAL, SDDMM_BAND = 0, 1, 2, 3


class SpmmProblem(C.Structure):
    """segtaco_spmm_problem: one SpMM of a batch (device pointers)."""
    _fields_ = [("M", C.c_int32), ("K", C.c_int32), ("N", C.c_int32), ("b_dtype", C.c_int32),
                ("nnz", C.c_int64), ("row_ptr", C.c_void_p), ("col", C.c_void_p),
                ("vals", C.c_void_p), ("B", C.c_void_p), ("ldb", C.c_int64), ("C", C.c_void_p),
                ("ldc", C.c_int64)]


OP_SPMM, OP_SDDMM = 0, 1
SERVER_PER_CALL, SERVER_FAKE_DEVICE = 1, 2
REQ_DEVICE_DENSE = 1


class ServerConfig(C.Structure):
    """segtaco_server_config: zero fields take the defaults."""
    _fields_ = [("max_batch", C.c_int32), ("slots", C.c_int32), ("cache_bytes", C.c_int64),
                ("staging_bytes", C.c_int64), ("reserve_bytes", C.c_int64),
                ("flags", C.c_uint32), ("fail_alloc_at", C.c_int32),
                ("fake_delay_us", C.c_int32), ("reserved", C.c_int32)]


class Request(C.Structure):
    """segtaco_request."""
    _fields_ = [("op", C.c_int32), ("dtype", C.c_int32), ("matrix", C.c_int64),
                ("N", C.c_int32), ("flags", C.c_uint32), ("B", C.c_void_p), ("Y", C.c_void_p),
                ("out", C.c_void_p)]


class ServerStats(C.Structure):
    """segtaco_server_stats."""
    _fields_ = [(f, C.c_int64) for f in (
        "submitted", "completed", "failed", "cancelled", "pending", "in_flight", "batches",
        "cache_hits", "cache_misses", "evictions", "cache_bytes", "h2d_bytes", "d2h_bytes")] + \
        [(f, C.c_double) for f in ("p50_us", "p99_us", "max_us", "mean_us", "span_s",
                                   "mean_batch")]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


MTX_SEGTACO_PATTERN = 1
MTX_VALUES_FILE, MTX_VALUES_SEGTACO, MTX_VALUES_ONES = 0, 1, 2


class HostCSR(C.Structure):
    """segtaco_host_csr (arrays malloc'd by the library)."""
    _fields_ = [("M", C.c_int32), ("K", C.c_int32), ("nnz", C.c_int64),
                ("row_ptr", C.POINTER(C.c_int32)), ("col", C.POINTER(C.c_int32)),
                ("vals", C.POINTER(C.c_float))]


class TacoTensor(C.Structure):
    """taco_tensor_t (segTACO taco_tensor_t.h:6-15), same layout."""
    _fields_ = [("order", C.c_int32), ("dimensions", C.POINTER(C.c_int32)),
                ("csize", C.c_int32), ("mode_ordering", C.POINTER(C.c_int32)),
                ("mode_types", C.c_void_p), ("indices", C.POINTER(C.POINTER(C.POINTER(C.c_int32)))),
                ("vals", C.POINTER(C.c_float)), ("vals_size", C.c_int32)]


# name -> (restype, argtypes) of every extern "C" function in include/*.h
_I, _I64, _P, _SZ = C.c_int32, C.c_int64, C.c_void_p, C.c_size_t
SIGNATURES = {
    "segtaco_version": (C.c_char_p, []),
    "segtaco_last_error": (C.c_char_p, []),
    "segtaco_device_available": (C.c_int, []),
    "segtaco_device_status": (C.c_int, [C.c_int]),
    "segtaco_autotune_heuristic": (C.c_int, [_I, _I, _I64, _I, _I, _I64, C.POINTER(Config)]),
    "segtaco_spmm_workspace_size": (C.c_int, [_I, _I, _I64, _I, _I, C.POINTER(Config),
                                              C.POINTER(_SZ)]),
    "segtaco_spmm": (C.c_int, [_I, _I, _I64, _P, _P, _P, _P, _I, _I64, _P, _I64, _I,
                               C.POINTER(Config), _P, _SZ, _P]),
    "segtaco_spmm_noalloc": (C.c_int, [_I, _I, _I64, _P, _P, _P, _P, _I, _I64, _P, _I64, _I,
                                       C.POINTER(Config), _P]),
    "segtaco_spmm_partition": (C.c_int, [_I, _I, _I64, _P, _P, _I64, _I, _I, C.POINTER(Config),
                                         _P, _SZ, _P]),
    "segtaco_vendor_spmm": (C.c_int, [_I, _I, _I64, _P, _P, _P, _P, _I64, _P, _I64, _I, _P]),
    "segtaco_batch_create": (C.c_int, [_I, C.POINTER(SpmmProblem), C.POINTER(Config), _P,
                                       C.POINTER(_P)]),
    "segtaco_batch_run": (C.c_int, [_P, _P]),
    "segtaco_batch_run_graph": (C.c_int, [_P, _P]),
    "segtaco_batch_run_gated": (C.c_int, [_P, _P, _I64, _P]),
    "segtaco_batch_info": (C.c_int, [_P, C.POINTER(_I), C.POINTER(_I64), C.POINTER(Config)]),
    "segtaco_batch_destroy": (C.c_int, [_P]),
    "segtaco_row_stats": (C.c_int, [_I, _P, C.POINTER(_I64), _P]),
    "segtaco_band_stats": (C.c_int, [_I, _I, _I64, _P, _P, _I, C.POINTER(_I64), _P]),
    "segtaco_spmm_plan_name": (C.c_int, [_I, _I, _I64, _I, _I, _P, _I64, _P, C.c_char_p,
                                         C.c_size_t]),
    "segtaco_server_create": (C.c_int, [C.POINTER(ServerConfig), C.POINTER(_P)]),
    "segtaco_server_add_matrix": (C.c_int, [_P, _I64, _I, _I, _I64, _P, _P, _P]),
    "segtaco_server_submit": (C.c_int, [_P, C.POINTER(Request), C.POINTER(_I64)]),
    "segtaco_server_replay": (C.c_int, [_P, _I, C.POINTER(Request), C.POINTER(C.c_double),
                                        C.POINTER(_I64)]),
    "segtaco_server_wait": (C.c_int, [_P, _I64, _I, C.POINTER(_I)]),
    "segtaco_server_drain": (C.c_int, [_P, _I]),
    "segtaco_server_cancel": (C.c_int, [_P, _I64]),
    "segtaco_server_get_stats": (C.c_int, [_P, _I, C.POINTER(ServerStats)]),
    "segtaco_server_destroy": (C.c_int, [_P]),
    "segtaco_probe_gather": (C.c_int, [_P, _I64, _I, _I64, C.c_uint32, _P, _I, _P]),
    "segtaco_probe_copy": (C.c_int, [_P, _P, _I64, _P, _I, _P]),
    "segtaco_mtx_read": (C.c_int, [C.c_char_p, C.c_uint32, _I, C.c_uint64, C.POINTER(HostCSR)]),
    "segtaco_host_csr_free": (None, [C.POINTER(HostCSR)]),
    "segtaco_block_starts_taco": (C.c_int, [_I, _I64, _P, _I, _P, _P]),
    "segtaco_block_starts_canonical": (C.c_int, [_I, _I64, _P, _I, _P, _P]),
    "segtaco_merge_path": (C.c_int, [_I, _I64, _P, _I64, _P, _P, _P]),
    "segtaco_row_ids": (C.c_int, [_I, _I64, _P, _P, _P]),
    "segtaco_csr_validate": (C.c_int, [_I, _I, _I64, _P, _P, _P]),
    "segtaco_spmv_workspace_size": (C.c_int, [_I, _I64, C.POINTER(_SZ)]),
    "segtaco_spmv": (C.c_int, [_I, _I, _I64, _P, _P, _P, _P, _P, _P, _SZ, _P]),
    "segtaco_sddmm": (C.c_int, [_I, _I, _I64, _P, _P, _P, _P, _P, _I, _I64, _I64, _I, _P, _P]),
    "segtaco_sddmm_autotune": (C.c_int, [_I, _I, _I64, _I, _I, _I64, C.POINTER(SddmmConfig)]),
    "segtaco_sddmm_ex": (C.c_int, [_I, _I, _I64, _P, _P, _P, _P, _P, _I, _I64, _I64, _I, _P,
                                   C.POINTER(SddmmConfig), _P]),
    "segtaco_spmspv": (C.c_int, [_I, _I, _I64, _P, _P, _P, _I, _P, _P, _P, _P]),
    "segtaco_taco_call": (C.c_int, [_P, C.POINTER(TacoTensor), C.POINTER(TacoTensor),
                                    C.POINTER(TacoTensor), C.POINTER(TacoTensor)]),
    "segtaco_taco_timer_ms": (C.c_float, []),
    "segtaco_taco_release": (None, []),
    "segtaco_taco_num_names": (C.c_int, []),
    "segtaco_taco_name": (C.c_char_p, [C.c_int]),
}

_lib = None


def lib():
    """Load libsegtaco.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise SegtacoError(EINVAL, "libsegtaco.so not built (run segtaco_gb300/build.py): %s"
                               % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def last_error() -> str:
    return lib().segtaco_last_error().decode()


def check(status: int) -> None:
    if status != OK:
        raise SegtacoError(status, last_error())


def version() -> str:
    return lib().segtaco_version().decode()


def device_available() -> bool:
    return bool(lib().segtaco_device_available())


def taco_names():
    L = lib()
    return [L.segtaco_taco_name(i).decode() for i in range(L.segtaco_taco_num_names())]
