"""Row blocks with their B window staged by TMA (SEGTACO_FLAG_WINDOW): the
same products as the row-block kernel, whatever share of the gathers the
window serves -- banded and scattered matrices, fp32 and bf16 B, slabs cut by
N, window heights, the top and bottom edges (rows outside B zero-filled by the
copy), strided and offset B; rb_sr stays bit-exact with the sequential FMA
order.  rb_pr with N >= 64 takes the band kernel (32-row blocks, the band of A
as a dense tile, off-band nonzeros gathered): the same cases against the FP64
oracle, halos 0..112, N not a multiple of the 64-column slab, rows past the
last block, matrices with no band at all."""
import numpy as np
import pytest
import torch

from gpu_util import assert_spmm_close, dev, to_torch_bf16
from oracle import oracle as O
from segtaco_gb300 import native as N
from segtaco_gb300 import ops, synth

pytestmark = pytest.mark.gpu


def _cfg(sched, rpu=16, halo=32, col_tile=0, vec=0, flags=N.FLAG_WINDOW):
    c = N.Config.make(schedule=sched, rows_per_unit=rpu, items_per_unit=halo, flags=flags)
    c.col_tile = col_tile
    c.vec = vec
    return c


def _spmm(Ad, Bd, cfg, kernel="window"):
    """The product through the window kernel, or for rb_pr with N >= 64 (a
    multiple of 16) and 16-byte aligned operands the band kernel (the plan
    must pick it)."""
    name = ops.plan_name(Ad, Bd, cfg)
    if kernel == "window" and cfg.schedule == N.RB_PR and " band " in name:
        kernel = "band"
    assert (" %s " % kernel) in name, name
    return ops.spmm(Ad, Bd, config=cfg)


BANDED = synth.banded_plus_random(3000, 32, 8, seed=41)
SHORT_BAND = synth.banded_plus_random(777, 5, 2, seed=42)


@pytest.mark.parametrize("n,col_tile,vec", [(64, 64, 8), (64, 32, 8), (64, 32, 4), (40, 32, 8),
                                            (128, 64, 8), (32, 32, 4), (96, 64, 4)])
@pytest.mark.parametrize("name", ["banded", "short_band"])
def test_window_rb_pr_fp32(cuda, name, n, col_tile, vec):
    A = {"banded": BANDED, "short_band": SHORT_BAND}[name]
    B = synth.dense(A.K, n, seed=43)
    C = _spmm(dev(A), torch.from_numpy(B).cuda(), _cfg(N.RB_PR, col_tile=col_tile, vec=vec))
    torch.cuda.synchronize()
    assert_spmm_close(C.cpu().numpy(), A, B)


@pytest.mark.parametrize("rpu,halo", [(1, 0), (4, 8), (16, 32), (16, 64), (32, 32), (8, 96)])
def test_window_heights(cuda, rpu, halo):
    B = synth.dense(BANDED.K, 64, seed=44)
    C = _spmm(dev(BANDED), torch.from_numpy(B).cuda(),
              _cfg(N.RB_PR, rpu=rpu, halo=halo, col_tile=64, vec=8))
    torch.cuda.synchronize()
    assert_spmm_close(C.cpu().numpy(), BANDED, B)


def test_window_rb_sr_bitexact(cuda):
    """rb_sr reads B from the window but keeps each column's storage-order chain."""
    A = BANDED
    B = synth.dense(A.K, 64, seed=45)
    want = O.spmm_f32_rowseq(A.row_ptr, A.col, A.val, B, fma=True)
    for col_tile in (32, 64):
        # rb_sr is one 32-lane slot: 1 or 2 columns per lane over 32 or 64 columns
        c = _cfg(N.RB_SR, col_tile=col_tile)
        C = _spmm(dev(A), torch.from_numpy(B).cuda(), c)
        torch.cuda.synchronize()
        assert np.array_equal(C.cpu().numpy(), want)


@pytest.mark.parametrize("n", [64, 128])
def test_window_bf16(cuda, n):
    A = BANDED
    Bf = synth.dense(A.K, n, seed=46)
    bits = synth.to_bf16_bits(Bf)
    Bw = synth.bf16_bits_to_f32(bits)
    C = _spmm(dev(A), to_torch_bf16(bits), _cfg(N.RB_PR, col_tile=64, vec=16))
    torch.cuda.synchronize()
    assert_spmm_close(C.cpu().numpy(), A, Bw)


@pytest.mark.parametrize("name", ["powerlaw", "rect", "half_empty"])
def test_window_scattered_and_rectangular(cuda, name):
    """Matrices whose gathers mostly miss the window (and K != M)."""
    A = {"powerlaw": synth.power_law(5000, 4000, 1.8, 1500, 0.02, seed=47),
         "rect": synth.random_csr(2000, 700, 0.03, seed=48),
         "half_empty": synth.random_csr(1500, 3100, 0.01, seed=49, p_empty=0.5)}[name]
    B = synth.dense(A.K, 64, seed=50)
    C = _spmm(dev(A), torch.from_numpy(B).cuda(), _cfg(N.RB_PR, col_tile=64, vec=8))
    torch.cuda.synchronize()
    assert_spmm_close(C.cpu().numpy(), A, B)


def test_window_strided_offset_b(cuda):
    """B a strided view (ldb > N) starting 16 bytes into its allocation."""
    A = BANDED
    big = torch.from_numpy(synth.dense(A.K, 80, seed=51)).cuda()
    Bv = big[:, 4:68]  # ldb 80, base 16 bytes in
    C = _spmm(dev(A), Bv, _cfg(N.RB_PR, col_tile=64, vec=4))
    torch.cuda.synchronize()
    assert_spmm_close(C.cpu().numpy(), A, Bv.cpu().numpy())


def test_window_overwrites_c(cuda):
    A = SHORT_BAND
    B = synth.dense(A.K, 64, seed=52)
    Cd = torch.full((A.M, 64), float("nan"), device="cuda")
    Ad, Bd = dev(A), torch.from_numpy(B).cuda()
    for c, kernel in ((_cfg(N.RB_PR, col_tile=64, vec=8), " band "),
                      (_cfg(N.RB_SR, col_tile=64), " window ")):
        assert kernel in ops.plan_name(Ad, Bd, c)
        Cd.fill_(float("nan"))
        ops.spmm(Ad, Bd, C_out=Cd, config=c)
        torch.cuda.synchronize()
        assert_spmm_close(Cd.cpu().numpy(), A, B)
    ops.spmm(Ad, Bd, C_out=Cd, config=c)
    torch.cuda.synchronize()
    assert_spmm_close(Cd.cpu().numpy(), A, B)


def test_band_stats_and_autotune(cuda):
    Ad = dev(BANDED)
    k = ops.band_stats(Ad, 32)
    assert k == int(round(ops.in_band_fraction_host(BANDED, 32) * BANDED.nnz))
    assert 2 * k >= BANDED.nnz
    P = synth.power_law(5000, 4000, 1.8, 1500, 0.02, seed=47)
    kp = ops.band_stats(dev(P), 32)  # rows of up to 1,500 nonzeros: one warp strides each
    assert kp == int(round(ops.in_band_fraction_host(P, 32) * P.nnz))
    assert 10 * kp < P.nnz
    # the autotuner measures the band and takes the band kernel for rb_pr
    # (N >= 64); the window for the row-block walk stays an explicit request
    c = ops.autotune(Ad, 64)
    assert c.schedule == N.RB_PR and c.flags & N.FLAG_WINDOW and c.items_per_unit == 32
    B = synth.dense(BANDED.K, 64, seed=53)
    C = _spmm(Ad, torch.from_numpy(B).cuda(), c, kernel="band")
    torch.cuda.synchronize()
    assert_spmm_close(C.cpu().numpy(), BANDED, B)
    assert not ops.autotune(Ad, 32).flags & N.FLAG_WINDOW  # N < 64: plain row blocks
    assert not ops.autotune(dev(P), 64).flags & N.FLAG_WINDOW  # no band


@pytest.mark.parametrize("n", [64, 128, 80, 96, 256])
@pytest.mark.parametrize("name", ["banded", "short_band", "powerlaw", "rect", "half_empty"])
def test_band_kernel(cuda, name, n):
    A = {"banded": BANDED, "short_band": SHORT_BAND,
         "powerlaw": synth.power_law(5000, 4000, 1.8, 1500, 0.02, seed=47),
         "rect": synth.random_csr(2000, 700, 0.03, seed=48),
         "half_empty": synth.random_csr(1500, 3100, 0.01, seed=49, p_empty=0.5)}[name]
    B = synth.dense(A.K, n, seed=54 + n)
    Cd = torch.full((A.M, n), float("nan"), device="cuda")
    Ad, Bd = dev(A), torch.from_numpy(B).cuda()
    c = N.Config.make(schedule=N.RB_PR, flags=N.FLAG_WINDOW)
    assert " band " in ops.plan_name(Ad, Bd, c), ops.plan_name(Ad, Bd, c)
    ops.spmm(Ad, Bd, C_out=Cd, config=c)
    torch.cuda.synchronize()
    assert_spmm_close(Cd.cpu().numpy(), A, B)


@pytest.mark.parametrize("halo", [0, 1, 8, 32, 64, 112])
def test_band_halos(cuda, halo):
    B = synth.dense(BANDED.K, 64, seed=55)
    c = N.Config.make(schedule=N.RB_PR, items_per_unit=halo, flags=N.FLAG_WINDOW)
    if halo == 0:
        c.items_per_unit = 0  # 0 = the default halo of 32
    C = _spmm(dev(BANDED), torch.from_numpy(B).cuda(), c, kernel="band")
    torch.cuda.synchronize()
    assert_spmm_close(C.cpu().numpy(), BANDED, B)


@pytest.mark.parametrize("n", [64, 128])
def test_band_bf16_strided_and_edges(cuda, n):
    """bf16 B; B a strided view 16 bytes into its allocation; 3,001 rows (a
    last block of one row); values all one (vals = NULL)."""
    A = synth.banded_plus_random(3001, 16, 4, seed=56)
    bits = synth.to_bf16_bits(synth.dense(A.K, n, seed=57))
    C = _spmm(dev(A), to_torch_bf16(bits), N.Config.make(schedule=N.RB_PR, flags=N.FLAG_WINDOW),
              kernel="band")
    torch.cuda.synchronize()
    assert_spmm_close(C.cpu().numpy(), A, bits, bf16=True)
    big = torch.from_numpy(synth.dense(A.K, n + 16, seed=58)).cuda()
    Bv = big[:, 4:4 + n]
    C = _spmm(dev(A), Bv, N.Config.make(schedule=N.RB_PR, flags=N.FLAG_WINDOW), kernel="band")
    torch.cuda.synchronize()
    assert_spmm_close(C.cpu().numpy(), A, Bv.cpu().numpy())
    ones = synth.CSR(A.row_ptr, A.col, np.ones_like(A.val), A.M, A.K)
    Ad = ops.DeviceCSR.from_host(ones, "cuda", with_values=False)
    B = synth.dense(A.K, n, seed=59)
    C = _spmm(Ad, torch.from_numpy(B).cuda(), N.Config.make(schedule=N.RB_PR, flags=N.FLAG_WINDOW),
              kernel="band")
    torch.cuda.synchronize()
    assert_spmm_close(C.cpu().numpy(), ones, B)


def _dup_csr(A, seed):
    """A with every 7th nonzero of each row repeated once (duplicate entries
    that must add up)."""
    rng = np.random.default_rng(seed)
    rows, cols, vals = [], [], []
    for r in range(A.M):
        s0, s1 = int(A.row_ptr[r]), int(A.row_ptr[r + 1])
        c = list(A.col[s0:s1])
        v = list(A.val[s0:s1])
        for k in range(0, s1 - s0, 7):
            c.append(A.col[s0 + k])
            v.append(np.float32(rng.uniform(-1, 1)))
        rows.append(len(c))
        cols += c
        vals += v
    rp = np.zeros(A.M + 1, np.int64)
    np.cumsum(rows, out=rp[1:])
    return synth.CSR(rp.astype(np.int32), np.array(cols, np.int32), np.array(vals, np.float32),
                     A.M, A.K)


@pytest.mark.parametrize("m,k,n", [(1, 1, 64), (1, 200, 64), (31, 31, 64), (33, 40, 80),
                                   (40, 40, 64), (97, 5, 64), (5, 3000, 128), (700, 90, 64)])
def test_band_kernel_small_shapes(cuda, m, k, n):
    """Tiny and ragged shapes: one row, one column, a last block of 1 row, K
    smaller than the 96-row window (the copy's rows past K zero-filled), tall
    and wide rectangles."""
    A = synth.random_csr(m, k, min(1.0, 12.0 / k), seed=m * 7 + k)
    B = synth.dense(k, n, seed=m + k)
    Ad, Bd = dev(A), torch.from_numpy(B).cuda()
    c = N.Config.make(schedule=N.RB_PR, flags=N.FLAG_WINDOW)
    assert " band " in ops.plan_name(Ad, Bd, c)
    Cd = torch.full((m, n), float("nan"), device="cuda")
    ops.spmm(Ad, Bd, C_out=Cd, config=c)
    torch.cuda.synchronize()
    assert_spmm_close(Cd.cpu().numpy(), A, B)


def test_band_kernel_duplicate_entries(cuda):
    """Duplicate (row, column) entries add up in the band tile and in the
    off-band lists."""
    A = _dup_csr(synth.banded_plus_random(600, 12, 3, seed=73), 74)
    B = synth.dense(A.K, 64, seed=75)
    C = _spmm(dev(A), torch.from_numpy(B).cuda(),
              N.Config.make(schedule=N.RB_PR, flags=N.FLAG_WINDOW), kernel="band")
    torch.cuda.synchronize()
    assert_spmm_close(C.cpu().numpy(), A, B)


def test_band_kernel_long_off_band_rows(cuda):
    """Rows with more off-band nonzeros than the per-row list holds (16) walk
    their nonzeros in global memory instead."""
    rng = np.random.default_rng(76)
    M = K = 2000
    keys = []
    for r in range(M):
        n_off = 40 if r % 5 == 0 else 3
        cs = set(range(max(0, r - 8), min(K, r + 9)))
        cs |= set(int(x) for x in rng.integers(0, K, n_off))
        keys.extend(r * K + np.array(sorted(cs), np.int64))
    A = synth._from_keys(np.array(keys, np.int64), M, K, rng)
    B = synth.dense(K, 64, seed=77)
    C = _spmm(dev(A), torch.from_numpy(B).cuda(),
              N.Config.make(schedule=N.RB_PR, flags=N.FLAG_WINDOW), kernel="band")
    torch.cuda.synchronize()
    assert_spmm_close(C.cpu().numpy(), A, B)
