"""Serving loop over the C ABI (segtaco_server_*).

The scheduler, the device CSR cache and the batching all run natively in
libsegtaco; this module only registers host arrays, builds request structs and
keeps the Python objects behind every pointer alive until the request is done.
"""
from __future__ import annotations

import ctypes as C
import threading

import numpy as np

from . import native as N


def _addr(a):
    """Address of a numpy array or a torch tensor (host or device)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        if not a.flags["C_CONTIGUOUS"]:
            raise N.SegtacoError(N.EINVAL, "operands must be C-contiguous")
        return a.ctypes.data
    return a.data_ptr()


def _dtype_of(a):
    name = str(a.dtype)
    if name in ("float32", "torch.float32"):
        return N.F32
    if name in ("uint16", "int16", "torch.bfloat16", "torch.int16"):
        return N.BF16  # bf16 bit patterns
    raise N.SegtacoError(N.EINVAL, "dense operand must be float32 or bf16 bits, got %s" % name)


class Server:
    """A running serving loop.  Matrices are registered once by id; requests
    name a matrix id and carry their dense operands (host arrays are staged by
    the server, device tensors are used in place with device=True)."""

    def __init__(self, max_batch=0, slots=0, cache_bytes=0, staging_bytes=0, reserve_bytes=0,
                 flags=0, fail_alloc_at=0, fake_delay_us=0):
        cfg = N.ServerConfig(max_batch, slots, cache_bytes, staging_bytes, reserve_bytes, flags,
                             fail_alloc_at, fake_delay_us, 0)
        h = C.c_void_p()
        N.check(N.lib().segtaco_server_create(C.byref(cfg), C.byref(h)))
        self._h = h
        self._mats = {}
        self._keep = {}
        self._mu = threading.Lock()

    # ---- matrices ----
    def add_matrix(self, mid: int, A, pin: bool = False):
        """Register CSR `A` (synth.CSR or any object with row_ptr, col, val, M, K)."""
        arrays = [np.ascontiguousarray(A.row_ptr, dtype=np.int32),
                  np.ascontiguousarray(A.col, dtype=np.int32),
                  None if A.val is None else np.ascontiguousarray(A.val, dtype=np.float32)]
        if pin:
            import torch
            arrays = [None if x is None else torch.from_numpy(x).pin_memory() for x in arrays]
        nnz = int(arrays[0][-1]) if A.M else 0
        N.check(N.lib().segtaco_server_add_matrix(self._h, mid, A.M, A.K, nnz,
                                                  _addr(arrays[0]), _addr(arrays[1]),
                                                  _addr(arrays[2])))
        self._mats[mid] = arrays

    # ---- requests ----
    @staticmethod
    def request(op, mid, B, out, Y=None, device=False, N_cols=None):
        r = N.Request()
        r.op = op
        r.matrix = mid
        r.dtype = _dtype_of(B)
        r.N = int(N_cols if N_cols is not None else B.shape[1])
        r.flags = N.REQ_DEVICE_DENSE if device else 0
        r.B = _addr(B)
        r.Y = _addr(Y)
        r.out = _addr(out)
        return r

    def submit_request(self, r, keep):
        t = C.c_int64()
        N.check(N.lib().segtaco_server_submit(self._h, C.byref(r), C.byref(t)))
        with self._mu:
            self._keep[t.value] = keep
        return t.value

    def spmm(self, mid, B, C_out, device=False):
        """Queue C_out = A[mid] @ B; returns the ticket."""
        return self.submit_request(self.request(N.OP_SPMM, mid, B, C_out, device=device),
                                   (B, C_out))

    def sddmm(self, mid, X, Y, out, device=False):
        """Queue out[p] = A.val[p] * <X[i], Y[j]> over the nonzeros of A[mid]."""
        return self.submit_request(self.request(N.OP_SDDMM, mid, X, out, Y=Y, device=device),
                                   (X, Y, out))

    def replay(self, requests, arrivals_us, keep=None):
        """Open-loop arrivals: request i is submitted arrivals_us[i] after the
        call starts (native thread timing).  Returns the tickets."""
        n = len(requests)
        arr = (N.Request * n)(*requests)
        times = (C.c_double * n)(*[float(t) for t in arrivals_us])
        tickets = (C.c_int64 * n)()
        st = N.lib().segtaco_server_replay(self._h, n, arr, times, tickets)
        out = list(tickets)
        with self._mu:
            for t in out:
                if t >= 0:
                    self._keep[t] = keep
        N.check(st)
        return out

    def wait(self, ticket, timeout_ms=-1):
        """Final status of the request (N.OK, N.ENOMEM, N.ECANCELLED, ...), or
        None if it is still running after timeout_ms."""
        st = C.c_int32()
        rc = N.lib().segtaco_server_wait(self._h, ticket, timeout_ms, C.byref(st))
        if rc == N.ETIMEOUT:
            return None
        N.check(rc)
        with self._mu:
            self._keep.pop(ticket, None)
        return st.value

    def drain(self, timeout_ms=-1):
        N.check(N.lib().segtaco_server_drain(self._h, timeout_ms))

    def cancel(self, ticket):
        return N.lib().segtaco_server_cancel(self._h, ticket)

    def stats(self, reset=False):
        s = N.ServerStats()
        N.check(N.lib().segtaco_server_get_stats(self._h, 1 if reset else 0, C.byref(s)))
        return s.as_dict()

    def close(self):
        if self._h:
            N.lib().segtaco_server_destroy(self._h)
            self._h = None
            self._keep.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
