"""MatrixMarket ingest (segtaco_mtx_read, native) -> synth.CSR.

`segtaco=True` reproduces the CSR pattern segTACO's read_mtx_file builds
(ds.h:183-268), including the cut of mirrored symmetric files at the header's
entry count; values: "segtaco" ({0, 0.1, 0.2} from a seeded generator, the
distribution of segTACO's fill_random, ds.h:270-274), "file" or "ones".
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import native as N
from .synth import CSR

_VALUES = {"file": N.MTX_VALUES_FILE, "segtaco": N.MTX_VALUES_SEGTACO, "ones": N.MTX_VALUES_ONES}


def read_mtx(path: str, segtaco: bool = False, values: str = "file", seed: int = 0) -> CSR:
    h = N.HostCSR()
    N.check(N.lib().segtaco_mtx_read(str(path).encode(), N.MTX_SEGTACO_PATTERN if segtaco else 0,
                                     _VALUES[values], seed, C.byref(h)))
    M, K = int(h.M), int(h.K)
    try:
        nnz = int(h.nnz)
        rp = np.ctypeslib.as_array(h.row_ptr, shape=(M + 1,)).copy()
        col = np.ctypeslib.as_array(h.col, shape=(max(nnz, 1),))[:nnz].copy()
        val = np.ctypeslib.as_array(h.vals, shape=(max(nnz, 1),))[:nnz].copy()
    finally:
        N.lib().segtaco_host_csr_free(C.byref(h))
    return CSR(rp, col, val, M, K)
