"""segtaco_spmm_noalloc: the SpMM entry point that allocates nothing.

It exists for callers that cannot call cudaMalloc (a framework whose own
allocator owns the device memory, a serving loop whose memory budget is fixed
at start-up): its scratch is a fixed array inside libsegtaco.  This file is
collected last so that a run stopping at the first failure has run every other
test first; it also passes alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from gpu_util import TOL, assert_spmm_close, dev, spmm_ref
from segtaco_gb300 import native as N
from segtaco_gb300 import ops, synth

pytestmark = pytest.mark.gpu


def _noalloc(Ad, Bd, Cd, cfg):
    p = lambda t: None if t is None else C.c_void_p(t.data_ptr())
    st = N.lib().segtaco_spmm_noalloc(Ad.M, Ad.K, Ad.nnz, p(Ad.row_ptr), p(Ad.col), p(Ad.val),
                                      p(Bd), N.F32, Bd.stride(0), p(Cd), Cd.stride(0),
                                      int(Bd.shape[1]), C.byref(cfg),
                                      C.c_void_p(torch.cuda.current_stream().cuda_stream))
    return st


@pytest.mark.parametrize("sched", ["eb_pr", "eb_sr"])
def test_noalloc_matches_spmm_twice(cuda, sched):
    A = synth.power_law(20000, 18000, 1.8, 5000, 0.02, seed=31)
    B = synth.dense(A.K, 64, seed=32)
    Ad, Bd = dev(A), torch.from_numpy(B).cuda()
    cfg = N.Config.make(schedule=sched, items_per_unit=256)
    ref_c = ops.spmm(Ad, Bd, config=cfg).cpu().numpy()  # the existing entry point
    ref = spmm_ref(A, B)
    for _ in range(2):  # the shared scratch keeps the previous call's contents
        Cd = torch.full((A.M, 64), float("nan"), device="cuda")
        assert _noalloc(Ad, Bd, Cd, cfg) == N.OK, N.last_error()
        torch.cuda.synchronize()
        got = Cd.cpu().numpy()
        assert_spmm_close(got, A, B, ref=ref)
        S = ref[1]
        assert np.all(np.abs(got - ref_c) <= 2 * TOL * np.maximum(S, 1e-30))


def test_noalloc_rejects_problems_beyond_its_scratch(cuda):
    # 300,000 rows of one nonzero at one item per chunk: 600,000 chunks, more
    # than twice the 262,143 the fixed scratch holds.
    M = 300_000
    rng = np.random.default_rng(33)
    row_ptr = np.arange(M + 1, dtype=np.int32)
    col = rng.integers(0, 1000, M, dtype=np.int32)
    Ad = dev(synth.CSR(row_ptr, col, np.ones(M, np.float32), M, 1000))
    Bd = torch.zeros((1000, 8), device="cuda")
    Cd = torch.zeros((M, 8), device="cuda")
    cfg = N.Config.make(schedule="eb_pr", items_per_unit=1)  # one chunk per item
    st = _noalloc(Ad, Bd, Cd, cfg)
    assert st == N.EINVAL and "fixed scratch" in N.last_error()


def test_noalloc_rb_sr_long_rows(cuda):
    """rb_sr from 1M nonzeros lists its long rows in the fixed scratch: the
    result stays the sequential FMA order, call after call."""
    from oracle import oracle as O
    A = synth.power_law(60_000, 50_000, 1.8, 40_000, 0.02, seed=35)
    assert A.nnz >= 1_000_000 and A.row_lengths().max() >= 2048
    # The long-row list (rows of >= 2048 nonzeros, two parts) fits the fixed
    # scratch, so the long-row CTAs run rather than the row-block fallback.
    hi, lo = A.nnz // (8 * 2048) + 1, A.nnz // 2048 + 1
    assert hi + lo <= 262144
    B = synth.dense(A.K, 128, seed=36)
    Ad, Bd = dev(A), torch.from_numpy(B).cuda()
    want = O.spmm_f32_rowseq(A.row_ptr, A.col, A.val, B, fma=True)
    cfg = N.Config.make(schedule="rb_sr", flags=N.FLAG_LONG_ROWS)
    for _ in range(2):
        Cd = torch.full((A.M, 128), float("nan"), device="cuda")
        assert _noalloc(Ad, Bd, Cd, cfg) == N.OK, N.last_error()
        torch.cuda.synchronize()
        assert np.array_equal(Cd.cpu().numpy(), want)


@pytest.mark.parametrize("n", [512, 128, 16])
def test_noalloc_rb_pr_long_rows(cuda, n):
    """rb_pr's long rows from 1M nonzeros: at N = 512 the pieces' partial rows
    (16 slabs of 32 columns) do not fit the fixed scratch and the long-row
    CTAs take them; at N = 128 and 16 they fit and the pieces run.  Within the
    FP64 bound and identical call after call either way."""
    A = synth.power_law(60_000, 50_000, 1.8, 40_000, 0.02, seed=35)
    assert A.nnz >= 1_000_000 and A.row_lengths().max() >= 512
    B = synth.dense(A.K, n, seed=37)
    Ad, Bd = dev(A), torch.from_numpy(B).cuda()
    cfg = N.Config.make(schedule="rb_pr", flags=N.FLAG_LONG_ROWS)
    ref = spmm_ref(A, B)
    first = None
    for _ in range(2):
        Cd = torch.full((A.M, n), float("nan"), device="cuda")
        assert _noalloc(Ad, Bd, Cd, cfg) == N.OK, N.last_error()
        torch.cuda.synchronize()
        got = Cd.cpu().numpy()
        assert_spmm_close(got, A, B, ref=ref)
        if first is None:
            first = got
        assert np.array_equal(got, first)
