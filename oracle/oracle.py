"""ctypes front end of the CPU oracle (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import
this module; the product library never does.  Every function wraps one C
function of ``segtaco_oracle.c`` / ``segtaco_cpu_baseline.c`` (see those files
for the segTACO source each one restates).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None

i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        L = C.CDLL(path)
        I, L64, V, D = C.c_int32, C.c_int64, C.c_void_p, C.c_double
        sig = {
            "orc_binary_search_segment_number": (I, [i32p, I, I, I]),
            "orc_taco_search_before": (I, [i32p, I, I, I]),
            "orc_taco_search_after": (I, [i32p, I, I, I]),
            "orc_block_starts_taco": (None, [i32p, I, I, I, i32p]),
            "orc_block_starts_canonical": (None, [i32p, I, I, I, i32p]),
            "orc_merge_path": (None, [i32p, I, L64, L64, L64, i32p, i32p]),
            "orc_row_ids": (None, [i32p, I, i32p]),
            "orc_spmm_f64": (None, [I, I, i32p, i32p, V, V, I, I, f64p, I]),
            "orc_spmm_absbound": (None, [I, I, i32p, i32p, V, V, I, I, f64p, I]),
            "orc_spmm_f32_rowseq": (None, [I, I, i32p, i32p, V, f32p, I, f32p, I, I]),
            "orc_spmv_f64": (None, [I, i32p, i32p, V, f32p, f64p]),
            "orc_sddmm_f64": (None, [I, I, i32p, i32p, V, V, V, I, I, I, f64p, V]),
            "orc_spmspv_f64": (None, [I, i32p, i32p, V, I, i32p, f32p, f64p, V]),
            "orc_max_bound_err_f32": (D, [L64, f32p, f64p, f64p]),
            "orc_max_rel_err_f32": (D, [L64, f32p, f64p, D]),
            "orc_num_threads": (I, []),
            "orc_cpu_spmm_eigen_order": (None, [I, I, i32p, i32p, f32p, f32p, f32p, I]),
            "orc_cpu_spmv_eigen_order": (None, [I, i32p, i32p, f32p, f32p, f32p, I]),
            "orc_cpu_threads": (I, []),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _vp(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


# ---- searches and partitions -------------------------------------------------

def binary_search_segment_number(row_ptr, M, nnz, e):
    return lib().orc_binary_search_segment_number(_c(row_ptr, np.int32), M + 0, nnz, e)


def taco_search_before(array, start, end, target):
    return lib().orc_taco_search_before(_c(array, np.int32), start, end, target)


def taco_search_after(array, start, end, target):
    return lib().orc_taco_search_after(_c(array, np.int32), start, end, target)


def block_starts_taco(row_ptr, M, P):
    row_ptr = _c(row_ptr, np.int32)
    nnz = int(row_ptr[M])
    nblk = (nnz + P - 1) // P
    out = np.empty(nblk + 1, np.int32)
    lib().orc_block_starts_taco(row_ptr, M, P, nblk, out)
    return out


def block_starts_canonical(row_ptr, M, P):
    row_ptr = _c(row_ptr, np.int32)
    nnz = int(row_ptr[M])
    nblk = (nnz + P - 1) // P
    out = np.empty(nblk + 1, np.int32)
    lib().orc_block_starts_canonical(row_ptr, M, P, nblk, out)
    return out


def merge_path(row_ptr, M, D):
    """(x, y) split of every chunk boundary for chunks of D merged items."""
    row_ptr = _c(row_ptr, np.int32)
    nnz = int(row_ptr[M])
    total = M + nnz
    nchunks = max(1, (total + D - 1) // D)
    xs = np.empty(nchunks + 1, np.int32)
    ys = np.empty(nchunks + 1, np.int32)
    lib().orc_merge_path(row_ptr, M, nnz, D, nchunks, xs, ys)
    return xs, ys


def row_ids(row_ptr, M):
    row_ptr = _c(row_ptr, np.int32)
    out = np.empty(int(row_ptr[M]), np.int32)
    lib().orc_row_ids(row_ptr, M, out)
    return out


# ---- products ----------------------------------------------------------------

def spmm_f64(row_ptr, col, val, B, bf16=False):
    """C = A B in double.  B is float32 (K, N) or, with bf16=True, uint16 bits."""
    row_ptr = _c(row_ptr, np.int32)
    col = _c(col, np.int32)
    val = None if val is None else _c(val, np.float32)
    B = np.ascontiguousarray(B)
    M = row_ptr.shape[0] - 1
    N = B.shape[1]
    out = np.empty((M, N), np.float64)
    lib().orc_spmm_f64(M, N, row_ptr, col, _vp(val), _vp(B), N, int(bf16), out, N)
    return out


def spmm_absbound(row_ptr, col, val, B, bf16=False):
    row_ptr = _c(row_ptr, np.int32)
    col = _c(col, np.int32)
    val = None if val is None else _c(val, np.float32)
    B = np.ascontiguousarray(B)
    M = row_ptr.shape[0] - 1
    N = B.shape[1]
    out = np.empty((M, N), np.float64)
    lib().orc_spmm_absbound(M, N, row_ptr, col, _vp(val), _vp(B), N, int(bf16), out, N)
    return out


def spmm_f32_rowseq(row_ptr, col, val, B, fma=False):
    """FP32 product in Eigen's row-major order (fma: fused multiply-add per step)."""
    row_ptr = _c(row_ptr, np.int32)
    col = _c(col, np.int32)
    val = None if val is None else _c(val, np.float32)
    B = _c(B, np.float32)
    M = row_ptr.shape[0] - 1
    N = B.shape[1]
    out = np.empty((M, N), np.float32)
    lib().orc_spmm_f32_rowseq(M, N, row_ptr, col, _vp(val), B, N, out, N, int(fma))
    return out


def spmv_f64(row_ptr, col, val, x):
    row_ptr = _c(row_ptr, np.int32)
    M = row_ptr.shape[0] - 1
    y = np.empty(M, np.float64)
    val = None if val is None else _c(val, np.float32)
    lib().orc_spmv_f64(M, row_ptr, _c(col, np.int32), _vp(val), _c(x, np.float32), y)
    return y


def sddmm_f64(row_ptr, col, val, X, Y, bf16=False):
    """out[p] = a_p * <X[i], Y[j]>; returns (out, bound)."""
    row_ptr = _c(row_ptr, np.int32)
    col = _c(col, np.int32)
    M = row_ptr.shape[0] - 1
    X = np.ascontiguousarray(X)
    Y = np.ascontiguousarray(Y)
    D = X.shape[1]
    nnz = int(row_ptr[M])
    val = None if val is None else _c(val, np.float32)
    out = np.empty(nnz, np.float64)
    bound = np.empty(nnz, np.float64)
    lib().orc_sddmm_f64(M, D, row_ptr, col, _vp(val), _vp(X), _vp(Y), D, D, int(bf16), out,
                        _vp(bound))
    return out, bound


def spmspv_f64(col_ptr, row_idx, val, M, x_idx, x_val):
    """y = A x with A given as CSC (col_ptr, row_idx, val) and x sparse."""
    col_ptr = _c(col_ptr, np.int32)
    y = np.empty(M, np.float64)
    bound = np.empty(M, np.float64)
    val = None if val is None else _c(val, np.float32)
    x_idx = _c(x_idx, np.int32)
    lib().orc_spmspv_f64(M, col_ptr, _c(row_idx, np.int32), _vp(val), x_idx.shape[0], x_idx,
                         _c(x_val, np.float32), y, _vp(bound))
    return y, bound


def max_bound_err(got, ref, S):
    got = _c(got, np.float32).reshape(-1)
    ref = _c(ref, np.float64).reshape(-1)
    S = _c(S, np.float64).reshape(-1)
    return lib().orc_max_bound_err_f32(got.shape[0], got, ref, S)


def max_rel_err(got, ref, floor_abs=0.0):
    got = _c(got, np.float32).reshape(-1)
    ref = _c(ref, np.float64).reshape(-1)
    return lib().orc_max_rel_err_f32(got.shape[0], got, ref, float(floor_abs))


# ---- the timed CPU baseline --------------------------------------------------

def cpu_spmm(row_ptr, col, val, B, out=None, threads=0):
    M = row_ptr.shape[0] - 1
    N = B.shape[1]
    if out is None:
        out = np.empty((M, N), np.float32)
    lib().orc_cpu_spmm_eigen_order(M, N, row_ptr, col, val, B, out, threads)
    return out


def cpu_spmv(row_ptr, col, val, x, out=None, threads=0):
    M = row_ptr.shape[0] - 1
    if out is None:
        out = np.empty(M, np.float32)
    lib().orc_cpu_spmv_eigen_order(M, row_ptr, col, val, x, out, threads)
    return out


def cpu_threads():
    return lib().orc_cpu_threads()
