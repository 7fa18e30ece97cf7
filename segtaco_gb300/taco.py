"""Host-side taco_tensor_t operands for the segTACO-named entry points.

Builds taco_tensor_t views (segTACO taco_tensor_t.h:6-15; CSR view as
ds.h:400-419, dense view as ds.h:432-444) over numpy arrays and calls a kernel
by its segTACO name through ``segtaco_taco_call``: the same path a segTACO
driver takes, with host buffers in and out.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import native as N


class _Holder:
    """Keeps the numpy arrays and ctypes objects behind one taco_tensor_t alive."""

    def __init__(self):
        self.keep = []

    def own(self, x):
        self.keep.append(x)
        return x


def dense(a: np.ndarray) -> tuple[N.TacoTensor, _Holder]:
    """Row-major dense matrix (or vector) view; writes land in `a`."""
    assert a.dtype == np.float32 and a.flags.c_contiguous
    h = _Holder()
    t = N.TacoTensor()
    dims = h.own((C.c_int32 * 2)(a.shape[0], a.shape[1] if a.ndim > 1 else 1))
    t.order = a.ndim
    t.dimensions = C.cast(dims, C.POINTER(C.c_int32))
    t.vals = a.ctypes.data_as(C.POINTER(C.c_float))
    h.own(a)
    return t, h


def csr(row_ptr, col, val, M, K) -> tuple[N.TacoTensor, _Holder]:
    h = _Holder()
    rp = h.own(np.ascontiguousarray(row_ptr, np.int32))
    cl = h.own(np.ascontiguousarray(col, np.int32))
    vv = h.own(np.ascontiguousarray(val, np.float32))
    t = N.TacoTensor()
    dims = h.own((C.c_int32 * 2)(M, K))
    t.order = 2
    t.dimensions = C.cast(dims, C.POINTER(C.c_int32))
    mode1 = h.own((C.POINTER(C.c_int32) * 2)(rp.ctypes.data_as(C.POINTER(C.c_int32)),
                                              cl.ctypes.data_as(C.POINTER(C.c_int32))))
    modes = h.own((C.POINTER(C.POINTER(C.c_int32)) * 2)(None, C.cast(mode1, C.POINTER(C.POINTER(C.c_int32)))))
    t.indices = C.cast(modes, C.POINTER(C.POINTER(C.POINTER(C.c_int32))))
    t.vals = vv.ctypes.data_as(C.POINTER(C.c_float))
    return t, h


def sparse_vector(idx, val, n) -> tuple[N.TacoTensor, _Holder]:
    """Sparse vector as segTACO's SpMSpV builds it: indices[0][0] = {0, nx},
    indices[0][1] = coordinates (spmspv_csr_gpu.h:53-72)."""
    h = _Holder()
    ix = h.own(np.ascontiguousarray(idx, np.int32))
    vv = h.own(np.ascontiguousarray(val, np.float32))
    pos = h.own(np.array([0, ix.shape[0]], np.int32))
    t = N.TacoTensor()
    dims = h.own((C.c_int32 * 1)(n))
    t.order = 1
    t.dimensions = C.cast(dims, C.POINTER(C.c_int32))
    mode0 = h.own((C.POINTER(C.c_int32) * 2)(pos.ctypes.data_as(C.POINTER(C.c_int32)),
                                              ix.ctypes.data_as(C.POINTER(C.c_int32))))
    modes = h.own((C.POINTER(C.POINTER(C.c_int32)) * 1)(C.cast(mode0, C.POINTER(C.POINTER(C.c_int32)))))
    t.indices = C.cast(modes, C.POINTER(C.POINTER(C.POINTER(C.c_int32))))
    t.vals = vv.ctypes.data_as(C.POINTER(C.c_float))
    return t, h


def call(name: str, out, a, b, c=None) -> float:
    """Run a segTACO-named kernel; returns the timed region in milliseconds."""
    L = N.lib()
    N.check(L.segtaco_taco_call(name.encode(), C.byref(out), C.byref(a), C.byref(b),
                                C.byref(c) if c is not None else None))
    return float(L.segtaco_taco_timer_ms())


def spmm(name: str, A, B: np.ndarray) -> tuple[np.ndarray, float]:
    """C = A B through the named entry point with host operands (A: synth.CSR-like)."""
    Cm = np.full((A.M, B.shape[1]), np.nan, np.float32)  # every element must be written
    tA, hA = csr(A.row_ptr, A.col, A.val, A.M, A.K)
    tB, hB = dense(np.ascontiguousarray(B, np.float32))
    tC, hC = dense(Cm)
    ms = call(name, tC, tA, tB)
    return Cm, ms
