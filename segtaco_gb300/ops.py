"""Device-level operations over the C ABI, with torch tensors as device memory.

torch only allocates device memory and names streams here; every computation
is a call into libsegtaco.so.  Tensors must be CUDA, contiguous (dense
operands may be row-strided), and index arrays int32.
"""
from __future__ import annotations

import ctypes as C
import dataclasses

import numpy as np
import torch

from . import native as N


def _ptr(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _stream(stream):
    if stream is None:
        stream = torch.cuda.current_stream()
    return C.c_void_p(stream.cuda_stream)


def _dense_dtype(t: torch.Tensor) -> int:
    if t.dtype == torch.float32:
        return N.F32
    if t.dtype == torch.bfloat16:
        return N.BF16
    raise N.SegtacoError(N.EINVAL, "dense operand must be float32 or bfloat16, got %s" % t.dtype)


@dataclasses.dataclass
class DeviceCSR:
    """A CSR matrix resident in device memory."""
    row_ptr: torch.Tensor
    col: torch.Tensor
    val: torch.Tensor | None
    M: int
    K: int

    @property
    def nnz(self) -> int:
        return int(self.col.shape[0])

    @classmethod
    def from_host(cls, csr, device="cuda", with_values=True):
        rp = torch.from_numpy(np.ascontiguousarray(csr.row_ptr, np.int32)).to(device)
        col = torch.from_numpy(np.ascontiguousarray(csr.col, np.int32)).to(device)
        val = None
        if with_values and csr.val is not None:
            val = torch.from_numpy(np.ascontiguousarray(csr.val, np.float32)).to(device)
        return cls(rp, col, val, int(csr.M), int(csr.K))

    def nbytes(self) -> int:
        n = self.row_ptr.numel() * 4 + self.col.numel() * 4
        return n + (0 if self.val is None else self.val.numel() * 4)


def spmm_workspace_size(A: DeviceCSR, n: int, b_dtype=N.F32, config: N.Config | None = None) -> int:
    out = C.c_size_t(0)
    N.check(N.lib().segtaco_spmm_workspace_size(A.M, A.K, A.nnz, n, b_dtype,
                                                C.byref(config) if config else None,
                                                C.byref(out)))
    return out.value


def spmm(A: DeviceCSR, B: torch.Tensor, C_out: torch.Tensor | None = None,
         config: N.Config | None = None, workspace: torch.Tensor | None = None,
         stream=None) -> torch.Tensor:
    """C = A @ B (B float32 or bfloat16, K x N row-major; C float32 M x N)."""
    if B.dim() != 2 or B.shape[0] != A.K:
        raise N.SegtacoError(N.EINVAL, "B must be K x N with K = %d" % A.K)
    n = int(B.shape[1])
    if C_out is None:
        C_out = torch.empty((A.M, n), dtype=torch.float32, device=B.device)
    ws_ptr, ws_bytes = None, 0
    if workspace is not None:
        ws_ptr, ws_bytes = _ptr(workspace), workspace.numel() * workspace.element_size()
    N.check(N.lib().segtaco_spmm(A.M, A.K, A.nnz, _ptr(A.row_ptr), _ptr(A.col), _ptr(A.val),
                                 _ptr(B), _dense_dtype(B), B.stride(0), _ptr(C_out),
                                 C_out.stride(0), n, C.byref(config) if config else None,
                                 ws_ptr, ws_bytes, _stream(stream)))
    return C_out


def vendor_spmm(A: DeviceCSR, B: torch.Tensor, C_out: torch.Tensor | None = None, stream=None):
    """cuSPARSE CSR_ALG2 on the same operands (comparator only)."""
    n = int(B.shape[1])
    if C_out is None:
        C_out = torch.empty((A.M, n), dtype=torch.float32, device=B.device)
    N.check(N.lib().segtaco_vendor_spmm(A.M, A.K, A.nnz, _ptr(A.row_ptr), _ptr(A.col), _ptr(A.val),
                                        _ptr(B), B.stride(0), _ptr(C_out), C_out.stride(0), n,
                                        _stream(stream)))
    return C_out


def spmm_partition(A: DeviceCSR, C_out: torch.Tensor, config: N.Config, workspace: torch.Tensor,
                   b_dtype=N.F32, stream=None) -> None:
    """First half of spmm(): partition + zeroing of split rows of C_out; follow
    with spmm(..., config with FLAG_PARTITION_READY, same workspace)."""
    N.check(N.lib().segtaco_spmm_partition(A.M, A.K, A.nnz, _ptr(A.row_ptr), _ptr(C_out),
                                           C_out.stride(0), int(C_out.shape[1]), b_dtype,
                                           C.byref(config), _ptr(workspace),
                                           workspace.numel() * workspace.element_size(),
                                           _stream(stream)))


def spmv_workspace_size(A: DeviceCSR) -> int:
    out = C.c_size_t()
    N.check(N.lib().segtaco_spmv_workspace_size(A.M, A.nnz, C.byref(out)))
    return out.value


def spmv(A: DeviceCSR, x: torch.Tensor, y: torch.Tensor | None = None,
         workspace: torch.Tensor | None = None, stream=None):
    """y = A @ x (fp32)."""
    if y is None:
        y = torch.empty(A.M, dtype=torch.float32, device=x.device)
    ws_ptr, ws_bytes = None, 0
    if workspace is not None:
        ws_ptr, ws_bytes = _ptr(workspace), workspace.numel() * workspace.element_size()
    N.check(N.lib().segtaco_spmv(A.M, A.K, A.nnz, _ptr(A.row_ptr), _ptr(A.col), _ptr(A.val),
                                 _ptr(x), _ptr(y), ws_ptr, ws_bytes, _stream(stream)))
    return y


def sddmm(A: DeviceCSR, X: torch.Tensor, Y: torch.Tensor, out: torch.Tensor | None = None,
          stream=None, config: "N.SddmmConfig | None" = None):
    """out[p] = A.val[p] * <X[i], Y[j]> over A's pattern (X: M x D, Y: K x D);
    config: a segtaco_sddmm_config (None: the library's choice)."""
    if out is None:
        out = torch.empty(A.nnz, dtype=torch.float32, device=X.device)
    dt = _dense_dtype(X)
    if _dense_dtype(Y) != dt:
        raise N.SegtacoError(N.EINVAL, "X and Y must have the same dtype")
    if config is None:
        N.check(N.lib().segtaco_sddmm(A.M, A.K, A.nnz, _ptr(A.row_ptr), _ptr(A.col),
                                      _ptr(A.val), _ptr(X), _ptr(Y), dt, X.stride(0),
                                      Y.stride(0), int(X.shape[1]), _ptr(out), _stream(stream)))
    else:
        N.check(N.lib().segtaco_sddmm_ex(A.M, A.K, A.nnz, _ptr(A.row_ptr), _ptr(A.col),
                                         _ptr(A.val), _ptr(X), _ptr(Y), dt, X.stride(0),
                                         Y.stride(0), int(X.shape[1]), _ptr(out), C.byref(config),
                                         _stream(stream)))
    return out


def sddmm_autotune(A, D: int, x_dtype=N.F32, max_row_len: int | None = None):
    """The library's SDDMM configuration (segtaco_sddmm_autotune) for A (a
    DeviceCSR: longest row and band statistics from the device; or a host
    CSR): the band kernel when at least half of the nonzeros lie within 32
    columns of the diagonal (D = 64)."""
    if isinstance(A, DeviceCSR):
        if max_row_len is None:
            max_row_len = int(row_stats(A)[0])
        banded = A.nnz > 0 and band_stats(A) * 2 >= A.nnz
    else:
        if max_row_len is None:
            max_row_len = int(np.diff(A.row_ptr).max()) if A.M > 0 else 0
        banded = A.nnz > 0 and in_band_fraction_host(A) >= 0.5
    cfg = N.SddmmConfig.make(N.SDDMM_BAND if banded else N.SDDMM_AUTO)
    N.check(N.lib().segtaco_sddmm_autotune(A.M, A.K, A.nnz, D, x_dtype, max_row_len,
                                           C.byref(cfg)))
    return cfg


def spmspv(At: DeviceCSR, x_idx: torch.Tensor, x_val: torch.Tensor, m: int,
           y: torch.Tensor | None = None, stream=None):
    """y = A x for sparse x; At is the CSR of A^T (At.M = columns of A), m = rows of A."""
    if y is None:
        y = torch.empty(m, dtype=torch.float32, device=x_val.device)
    N.check(N.lib().segtaco_spmspv(m, At.M, At.nnz, _ptr(At.row_ptr), _ptr(At.col), _ptr(At.val),
                                   int(x_idx.shape[0]), _ptr(x_idx), _ptr(x_val), _ptr(y),
                                   _stream(stream)))
    return y


def block_starts_taco(A: DeviceCSR, P: int, stream=None):
    out = torch.empty((A.nnz + P - 1) // P + 1, dtype=torch.int32, device=A.row_ptr.device)
    N.check(N.lib().segtaco_block_starts_taco(A.M, A.nnz, _ptr(A.row_ptr), P, _ptr(out),
                                              _stream(stream)))
    return out


def block_starts_canonical(A: DeviceCSR, P: int, stream=None):
    out = torch.empty((A.nnz + P - 1) // P + 1, dtype=torch.int32, device=A.row_ptr.device)
    N.check(N.lib().segtaco_block_starts_canonical(A.M, A.nnz, _ptr(A.row_ptr), P, _ptr(out),
                                                   _stream(stream)))
    return out


def merge_path(A: DeviceCSR, D: int, stream=None):
    nch = max(1, (A.M + A.nnz + D - 1) // D)
    xs = torch.empty(nch + 1, dtype=torch.int32, device=A.row_ptr.device)
    ys = torch.empty(nch + 1, dtype=torch.int32, device=A.row_ptr.device)
    N.check(N.lib().segtaco_merge_path(A.M, A.nnz, _ptr(A.row_ptr), D, _ptr(xs), _ptr(ys),
                                       _stream(stream)))
    return xs, ys


def row_ids(A: DeviceCSR, stream=None):
    out = torch.empty(max(1, A.nnz), dtype=torch.int32, device=A.row_ptr.device)
    N.check(N.lib().segtaco_row_ids(A.M, A.nnz, _ptr(A.row_ptr), _ptr(out), _stream(stream)))
    return out[: A.nnz]


def csr_validate(A: DeviceCSR, stream=None):
    """Raises SegtacoError(EINVAL) if the device CSR is malformed."""
    N.check(N.lib().segtaco_csr_validate(A.M, A.K, A.nnz, _ptr(A.row_ptr), _ptr(A.col),
                                         _stream(stream)))


def probe_gather(buf: torch.Tensor, row_bytes: int, n: int, blocks: int, seed: int = 0,
                 sink: torch.Tensor | None = None, stream=None):
    """Enqueue n random row gathers of row_bytes over device buffer `buf`."""
    nbytes = buf.numel() * buf.element_size()
    if sink is None:
        sink = torch.zeros(32, dtype=torch.float32, device=buf.device)
    N.check(N.lib().segtaco_probe_gather(C.c_void_p(buf.data_ptr()), nbytes // row_bytes,
                                         row_bytes, n, seed, C.c_void_p(sink.data_ptr()), blocks,
                                         _stream(stream)))
    return sink


def row_stats(A: DeviceCSR, stream=None):
    """Row-length statistics: (max length, empty rows, rows >= 32, nonzeros in rows >= 32)."""
    out = (C.c_int64 * 4)()
    N.check(N.lib().segtaco_row_stats(A.M, _ptr(A.row_ptr), out, _stream(stream)))
    return tuple(out)


def plan_name(A: DeviceCSR, B: torch.Tensor, config: N.Config | None = None) -> str:
    """The kernel plan segtaco_spmm picks for A @ B (segtaco_spmm_plan_name)."""
    buf = C.create_string_buffer(256)
    N.check(N.lib().segtaco_spmm_plan_name(A.M, A.K, A.nnz, int(B.shape[1]), _dense_dtype(B),
                                           C.c_void_p(B.data_ptr()), B.stride(0),
                                           C.byref(config) if config is not None else None,
                                           buf, 256))
    return buf.value.decode()


def band_stats(A: DeviceCSR, halo: int = 32, stream=None) -> int:
    """Nonzeros of A within `halo` columns of the diagonal (segtaco_band_stats)."""
    out = C.c_int64()
    N.check(N.lib().segtaco_band_stats(A.M, A.K, A.nnz, _ptr(A.row_ptr),
                                       _ptr(A.col) if A.nnz else None, halo, C.byref(out),
                                       _stream(stream)))
    return out.value


def in_band_fraction_host(A, halo: int = 32) -> float:
    """The same statistic from a host CSR."""
    if A.nnz == 0:
        return 0.0
    rows = np.repeat(np.arange(A.M, dtype=np.int64), np.diff(A.row_ptr))
    d = rows * A.K // max(A.M, 1)
    return float(np.count_nonzero(np.abs(A.col.astype(np.int64) - d) <= halo)) / A.nnz


def autotune(A, n: int, b_dtype=N.F32, schedule=N.AUTO, max_row_len: int | None = None):
    """The library's configuration for C = A @ B with n columns
    (segtaco_autotune_heuristic): the schedule (AUTO: row-balanced for even
    rows, merge path otherwise), slab, lanes, units; for row-balanced
    schedules from 1M nonzeros on, long rows out of the row blocks (rb_sr:
    rows of >= 2048 nonzeros to CTAs of their own; rb_pr: rows of >= 512 as
    pieces of 4096); and, when at least half of the nonzeros lie within 32 columns of
    the diagonal, rb_pr's band kernel (N >= 64, a multiple of 16).  `A` is a DeviceCSR
    (statistics from segtaco_row_stats / segtaco_band_stats on the device) or
    a host CSR (from its arrays), unless max_row_len is given."""
    banded = False
    if isinstance(A, DeviceCSR):
        if max_row_len is None:
            max_row_len = int(row_stats(A)[0])
        banded = A.nnz > 0 and band_stats(A) * 2 >= A.nnz
    else:
        if max_row_len is None:
            max_row_len = int(np.diff(A.row_ptr).max()) if A.M > 0 else 0
        banded = A.nnz > 0 and in_band_fraction_host(A) >= 0.5
    cfg = N.Config.make(schedule=schedule)
    if banded:
        cfg.flags = N.FLAG_WINDOW
    N.check(N.lib().segtaco_autotune_heuristic(A.M, A.K, A.nnz, n, b_dtype, max_row_len,
                                               C.byref(cfg)))
    return cfg


class Batch:
    """Many SpMMs planned together and run by one persistent launch per kernel
    variant (segtaco_batch_*).  `items` is a list of (DeviceCSR, B, C) with B
    fp32 or bf16 (K x N) and C fp32 (M x N); configs=None autotunes each."""

    def __init__(self, items, configs=None, stream=None):
        self._keep = list(items)
        probs = (N.SpmmProblem * len(items))()
        for p, (A, B, Cm) in zip(probs, items):
            p.M, p.K, p.N = A.M, A.K, int(B.shape[1])
            p.b_dtype = _dense_dtype(B)
            p.nnz = A.nnz
            p.row_ptr = A.row_ptr.data_ptr()
            p.col = A.col.data_ptr() if A.nnz else None
            p.vals = A.val.data_ptr() if A.val is not None else None
            p.B = B.data_ptr()
            p.ldb = B.stride(0)
            p.C = Cm.data_ptr()
            p.ldc = Cm.stride(0)
        cfgs = None
        if configs is not None:
            cfgs = (N.Config * len(items))(*configs)
        h = C.c_void_p()
        N.check(N.lib().segtaco_batch_create(len(items), probs, cfgs, _stream(stream), C.byref(h)))
        self._h = h
        self.count = len(items)

    def run(self, stream=None, graph=False):
        fn = N.lib().segtaco_batch_run_graph if graph else N.lib().segtaco_batch_run
        N.check(fn(self._h, _stream(stream)))

    def run_gated(self, gate: torch.Tensor, timeout_s: float = 1.0, stream=None):
        """Run with problems released by `gate` (int64 device tensor, or pinned
        host tensor): problem i runs once gate[0] > i."""
        N.check(N.lib().segtaco_batch_run_gated(self._h, C.c_void_p(gate.data_ptr()),
                                                int(timeout_s * 1e9), _stream(stream)))

    def info(self):
        g = C.c_int32()
        it = C.c_int64()
        cfgs = (N.Config * max(1, self.count))()
        N.check(N.lib().segtaco_batch_info(self._h, C.byref(g), C.byref(it), cfgs))
        return g.value, it.value, [cfgs[i] for i in range(self.count)]

    def close(self):
        if self._h:
            N.lib().segtaco_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
