"""Long rows of the row-block schedules.  From 1M nonzeros on, rows of at
least items_per_unit (default 2048) nonzeros are summed by CTAs of their own
that stage B row segments in shared memory, beside the row-block kernel on a
forked stream (FLAG_LONG_ROWS).  rb_sr: every column stays one fmaf chain in
storage order, so the result must be bit-identical to the one-warp walk
(without the flag) and to the sequential FP32 FMA restatement of segTACO's serial row sum
(spmm_rb_sr.h:187-243): across thresholds, widths (one and several column
slabs, widths the 16-byte copies cannot take), bf16 B, unit values, offset B,
the partition-ready split, and graph capture (the allocation-free entry point:
test_zz_no_alloc.py).  rb_pr: the long rows are pieces of 4096 nonzeros in
the row-block launch (over the same column slabs), whose partial rows the
last piece of each row sums in piece order: within the FP64 bound of 1e-5 and
bit-identical from run to run."""
import numpy as np
import pytest
import torch

from gpu_util import assert_spmm_close, dev, spmm_ref, to_torch_bf16
from oracle import oracle as O
from segtaco_gb300 import native as N
from segtaco_gb300 import ops, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def A():
    """Short rows (~29 nonzeros, 10 % empty) plus rows of exactly 50,000 /
    20,000 / 5,000 / 1,000 / 600 nonzeros, rows of 2047, 2048 and 2049 (the
    default threshold's edge), of 4095 / 4096 / 4097 and 8192 / 8193 (rb_pr's
    piece length and its double) and of 16,383 / 16,384 (where rows move to
    the front of the work list); 1.1M nonzeros."""
    rng = np.random.default_rng(41)
    M, K = 41_000, 50_000
    lengths = rng.binomial(64, 0.45, M)
    lengths[rng.random(M) < 0.1] = 0
    long_rows = {7: 50_000, 100: 20_000, 2_000: 5_000, 39_999: 600, 15_000: 2_047,
                 15_001: 2_048, 15_002: 2_049, 0: 1_000, 30_000: 16_383, 30_001: 16_384,
                 20_000: 4_095, 20_001: 4_096, 20_002: 4_097, 25_000: 8_192, 25_001: 8_193}
    for r in long_rows:
        lengths[r] = 0
    rows = np.repeat(np.arange(M, dtype=np.int64), lengths)
    keys = [np.unique(rows * K + rng.integers(0, K, rows.size))]
    keys += [r * K + np.sort(rng.choice(K, L, replace=False)) for r, L in long_rows.items()]
    A = synth._from_keys(np.sort(np.concatenate(keys)), M, K, rng)
    L = A.row_lengths()
    assert A.nnz >= 1_000_000 and all(L[r] == n for r, n in long_rows.items())
    return A


def rowseq(A, B, val=None):
    return O.spmm_f32_rowseq(A.row_ptr, A.col, A.val if val is None else val, B, fma=True)


def run(Ad, Bd, n, schedule="rb_sr", long=True, **kw):
    kw["flags"] = kw.get("flags", 0) | (N.FLAG_LONG_ROWS if long else 0)
    C_ = torch.full((Ad.M, n), float("nan"), device="cuda")
    ops.spmm(Ad, Bd, C_out=C_, config=N.Config.make(schedule=schedule, **kw))
    torch.cuda.synchronize()
    return C_.cpu().numpy()


@pytest.mark.parametrize("n", [128, 96, 64, 32, 8, 200, 126])
def test_bit_identical_to_one_warp_walk(cuda, A, n):
    B = synth.dense(A.K, n, seed=n)
    Ad, Bd = dev(A), torch.from_numpy(B).cuda()
    got = run(Ad, Bd, n)
    assert np.array_equal(got, run(Ad, Bd, n, long=False))
    assert np.array_equal(got, rowseq(A, B))


@pytest.mark.parametrize("threshold", [1, 31, 512, 2_049, 5_000, 10**7])
def test_thresholds(cuda, A, threshold):
    B = synth.dense(A.K, 64, seed=3)
    got = run(dev(A), torch.from_numpy(B).cuda(), 64, items_per_unit=threshold)
    assert np.array_equal(got, rowseq(A, B))


@pytest.mark.parametrize("n", [128, 64, 200])
def test_bf16_dense_operand(cuda, A, n):
    bits = synth.to_bf16_bits(synth.dense(A.K, n, seed=5))
    Bf = (bits.astype(np.uint32) << 16).view(np.float32)  # the bf16 values, exactly
    Ad, Bd = dev(A), to_torch_bf16(bits)
    got = run(Ad, Bd, n)
    assert np.array_equal(got, run(Ad, Bd, n, long=False))
    assert np.array_equal(got, rowseq(A, Bf))


def test_values_default_to_one(cuda, A):
    B = synth.dense(A.K, 64, seed=6)
    got = run(dev(A, with_values=False), torch.from_numpy(B).cuda(), 64)
    assert np.array_equal(got, rowseq(A, B, np.ones_like(A.val)))


@pytest.mark.parametrize("off", [4, 1])  # 16-byte aligned (long-row CTAs) and not
def test_offset_dense_operand(cuda, A, off):
    B = synth.dense(A.K, 64 + 8, seed=7)
    Bd = torch.from_numpy(B).cuda()[:, off:off + 64]
    got = run(dev(A), Bd, 64)
    assert np.array_equal(got, rowseq(A, np.ascontiguousarray(B[:, off:off + 64])))


def test_partition_ready_and_reruns(cuda, A):
    """segtaco_spmm_partition lists the long rows once; products with
    PARTITION_READY reuse the list (the work queue is cleared per launch)."""
    B = synth.dense(A.K, 128, seed=8)
    Ad, Bd = dev(A), torch.from_numpy(B).cuda()
    cfg = N.Config.make(schedule="rb_sr", flags=N.FLAG_LONG_ROWS)
    ws = torch.empty(ops.spmm_workspace_size(Ad, 128, N.F32, cfg), dtype=torch.uint8,
                     device="cuda")
    assert ws.numel() > 0
    C_ = torch.full((A.M, 128), float("nan"), device="cuda")
    ops.spmm_partition(Ad, C_, cfg, ws)
    ready = N.Config.make(schedule="rb_sr", flags=N.FLAG_LONG_ROWS | N.FLAG_PARTITION_READY)
    want = rowseq(A, B)
    for _ in range(3):
        C_.fill_(float("nan"))
        ops.spmm(Ad, Bd, C_out=C_, config=ready, workspace=ws)
        torch.cuda.synchronize()
        assert np.array_equal(C_.cpu().numpy(), want)


def test_graph_capture(cuda, A):
    """The fork to the side stream inside a captured graph, replayed."""
    B = synth.dense(A.K, 128, seed=9)
    Ad, Bd = dev(A), torch.from_numpy(B).cuda()
    cfg = N.Config.make(schedule="rb_sr", flags=N.FLAG_LONG_ROWS)
    ws = torch.empty(ops.spmm_workspace_size(Ad, 128, N.F32, cfg), dtype=torch.uint8,
                     device="cuda")
    C_ = torch.empty((A.M, 128), device="cuda")
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        ops.spmm(Ad, Bd, C_out=C_, config=cfg, workspace=ws)  # creates the side stream
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        ops.spmm(Ad, Bd, C_out=C_, config=cfg, workspace=ws)
    want = rowseq(A, B)
    for _ in range(2):
        C_.fill_(float("nan"))
        g.replay()
        torch.cuda.synchronize()
        assert np.array_equal(C_.cpu().numpy(), want)



@pytest.mark.parametrize("n", [128, 96, 64, 32, 8, 200, 126])
def test_rb_pr_long_rows(cuda, A, n):
    B = synth.dense(A.K, n, seed=50 + n)
    Ad, Bd = dev(A), torch.from_numpy(B).cuda()
    ref = spmm_ref(A, B)
    got = run(Ad, Bd, n, "rb_pr")
    assert_spmm_close(got, A, B, ref=ref)
    assert np.array_equal(got, run(Ad, Bd, n, "rb_pr"))  # no atomics: identical reruns
    assert_spmm_close(run(Ad, Bd, n, "rb_pr", long=False), A, B, ref=ref)


@pytest.mark.parametrize("threshold", [1, 512, 2_049])
def test_rb_pr_thresholds_and_bf16(cuda, A, threshold):
    bits = synth.to_bf16_bits(synth.dense(A.K, 64, seed=60))
    got = run(dev(A), to_torch_bf16(bits), 64, "rb_pr", items_per_unit=threshold)
    assert_spmm_close(got, A, bits, bf16=True)
    B = synth.dense(A.K, 128, seed=61)
    got = run(dev(A), torch.from_numpy(B).cuda(), 128, "rb_pr", items_per_unit=threshold)
    assert_spmm_close(got, A, B)


def test_rb_pr_pieces_partition_ready_and_graph(cuda, A):
    """rb_pr's long rows as pieces of the row-block launch: the plan names
    them; a list made once serves repeated products (each row's piece
    counters return to zero when its last piece has summed the partial rows),
    and a captured graph replays; every result is bit-identical (the partial
    rows are summed in piece order, whichever piece finishes last)."""
    B = synth.dense(A.K, 128, seed=62)
    Ad, Bd = dev(A), torch.from_numpy(B).cuda()
    cfg = N.Config.make(schedule="rb_pr", flags=N.FLAG_LONG_ROWS)
    assert ops.plan_name(Ad, Bd, cfg).startswith("rb_pr pieces ")
    ws = torch.empty(ops.spmm_workspace_size(Ad, 128, N.F32, cfg), dtype=torch.uint8,
                     device="cuda")
    C_ = torch.full((A.M, 128), float("nan"), device="cuda")
    ops.spmm_partition(Ad, C_, cfg, ws)
    ready = N.Config.make(schedule="rb_pr", flags=N.FLAG_LONG_ROWS | N.FLAG_PARTITION_READY)
    first = None
    for _ in range(3):
        C_.fill_(float("nan"))
        ops.spmm(Ad, Bd, C_out=C_, config=ready, workspace=ws)
        torch.cuda.synchronize()
        got = C_.cpu().numpy()
        if first is None:
            first = got
            assert_spmm_close(got, A, B)
        assert np.array_equal(got, first)
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        ops.spmm(Ad, Bd, C_out=C_, config=cfg, workspace=ws)
    for _ in range(2):
        C_.fill_(float("nan"))
        g.replay()
        torch.cuda.synchronize()
        assert np.array_equal(C_.cpu().numpy(), first)


@pytest.mark.parametrize("threshold,n", [(1, 64), (300, 40), (513, 128), (1024, 96),
                                         (4096, 128), (4097, 72)])
def test_rb_pr_pieces_one_and_several(cuda, A, threshold, n):
    """Thresholds below, at and above the piece length (4096): rows of one
    piece (stored directly) beside rows of several, ragged widths; identical
    reruns."""
    B = synth.dense(A.K, n, seed=63 + n)
    Ad, Bd = dev(A), torch.from_numpy(B).cuda()
    cfg = dict(items_per_unit=threshold)
    got = run(Ad, Bd, n, "rb_pr", **cfg)
    assert_spmm_close(got, A, B)
    assert np.array_equal(got, run(Ad, Bd, n, "rb_pr", **cfg))


@pytest.mark.parametrize("col_tile", [64, 32])
def test_rb_sr_narrow_slabs_bit_identical(cuda, A, col_tile):
    """rb_sr at 64- and 32-column slabs (N = 128): the long-row CTAs take the
    row blocks' slab width and the back part of their list slab by slab; every
    column is still one fmaf chain in storage order."""
    B = synth.dense(A.K, 128, seed=80)
    Ad, Bd = dev(A), torch.from_numpy(B).cuda()
    got = run(Ad, Bd, 128, "rb_sr", col_tile=col_tile)
    assert np.array_equal(got, rowseq(A, B))


def _with_long_rows_shuffled(A, seed):
    """A copy of A whose rows of >= 512 nonzeros hold their (column, value)
    pairs in a random order (CSR does not require sorted columns)."""
    rng = np.random.default_rng(seed)
    col, val = A.col.copy(), A.val.copy()
    rp = A.row_ptr
    for r in np.nonzero(A.row_lengths() >= 512)[0]:
        p = rng.permutation(rp[r + 1] - rp[r]) + rp[r]
        col[rp[r]:rp[r + 1]] = A.col[p]
        val[rp[r]:rp[r + 1]] = A.val[p]
    return synth.CSR(A.row_ptr, col, val, A.M, A.K)


@pytest.mark.parametrize("parts,n", [(2, 128), (3, 64), (8, 40), (2, 200), (5, 96)])
def test_rb_pr_pieces_in_passes(cuda, A, parts, n):
    """rb_pr's pieces in k_parts passes over ranges of B's rows (a launch of
    their own before the row blocks): every (piece, pass) leaves a partial row,
    summed in order, so reruns are bit-identical; thresholds that make rows of
    one piece (stored through the partials too) and of several."""
    B = synth.dense(A.K, n, seed=90 + parts)
    Ad, Bd = dev(A), torch.from_numpy(B).cuda()
    ref = spmm_ref(A, B)
    for threshold in (0, 300, 4097):
        cfg = dict(items_per_unit=threshold, k_parts=parts)
        assert ops.plan_name(Ad, Bd, N.Config.make(schedule="rb_pr", flags=N.FLAG_LONG_ROWS,
                                                   **cfg)).endswith(" parts=%d" % parts)
        got = run(Ad, Bd, n, "rb_pr", **cfg)
        assert_spmm_close(got, A, B, ref=ref)
        assert np.array_equal(got, run(Ad, Bd, n, "rb_pr", **cfg))


def test_rb_pr_pieces_in_passes_bf16_and_unsorted(cuda, A):
    """bf16 B in two passes; long rows with unsorted columns (each pass's range
    of a piece then holds columns of every range: still every nonzero once)."""
    bits = synth.to_bf16_bits(synth.dense(A.K, 64, seed=95))
    got = run(dev(A), to_torch_bf16(bits), 64, "rb_pr", k_parts=2)
    assert_spmm_close(got, A, bits, bf16=True)
    U = _with_long_rows_shuffled(A, 96)
    B = synth.dense(U.K, 128, seed=97)
    Ud, Bd = dev(U), torch.from_numpy(B).cuda()
    for parts in (2, 4):
        got = run(Ud, Bd, 128, "rb_pr", k_parts=parts)
        assert_spmm_close(got, U, B)
        assert np.array_equal(got, run(Ud, Bd, 128, "rb_pr", k_parts=parts))


def test_rb_pr_pieces_in_passes_one_sided_rows(cuda):
    """Long rows whose columns all fall in one pass's range (the other passes
    see an empty range and leave zero partial rows), one across a range edge
    and one starting exactly on it, a short row of that edge column alone, and
    K not a multiple of the pass count; partition-ready reruns and a graph
    replay."""
    rng = np.random.default_rng(98)
    M, K = 30_000, 10_007
    lengths = rng.binomial(70, 0.5, M)
    rows = np.repeat(np.arange(M, dtype=np.int64), lengths)
    keys = [np.unique(rows * K + rng.integers(0, K, rows.size))]
    edge = (K + 2) // 3  # the first column of pass 1 of 3
    special = {5: np.arange(0, 3000), 6: np.arange(K - 2500, K), 7: np.arange(edge - 700, edge + 700),
               8: np.array([edge]), 9: np.arange(edge, edge + 2000)}
    for r in special:
        keys[0] = keys[0][keys[0] // K != r]
    keys += [r * K + c for r, c in special.items()]
    A = synth._from_keys(np.sort(np.concatenate(keys)), M, K, rng)
    assert A.nnz >= 1_000_000
    B = synth.dense(K, 96, seed=99)
    Ad, Bd = dev(A), torch.from_numpy(B).cuda()
    ref = spmm_ref(A, B)
    cfg = N.Config.make(schedule="rb_pr", flags=N.FLAG_LONG_ROWS, k_parts=3)
    ws = torch.empty(ops.spmm_workspace_size(Ad, 96, N.F32, cfg), dtype=torch.uint8,
                     device="cuda")
    C_ = torch.full((A.M, 96), float("nan"), device="cuda")
    ops.spmm_partition(Ad, C_, cfg, ws)
    ready = N.Config.make(schedule="rb_pr", flags=N.FLAG_LONG_ROWS | N.FLAG_PARTITION_READY,
                          k_parts=3)
    first = None
    for _ in range(3):
        C_.fill_(float("nan"))
        ops.spmm(Ad, Bd, C_out=C_, config=ready, workspace=ws)
        torch.cuda.synchronize()
        got = C_.cpu().numpy()
        if first is None:
            first = got
            assert_spmm_close(got, A, B, ref=ref)
        assert np.array_equal(got, first)
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        ops.spmm(Ad, Bd, C_out=C_, config=cfg, workspace=ws)
    for _ in range(2):
        C_.fill_(float("nan"))
        g.replay()
        torch.cuda.synchronize()
        assert np.array_equal(C_.cpu().numpy(), first)
