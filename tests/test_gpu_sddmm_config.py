"""SDDMM configurations (segtaco_sddmm_ex / segtaco_sddmm_autotune): every
kernel, block size and lane count against the FP64 oracle, and the
autotuner's choice on the banded SDDMM configuration at full size and on
power-law rows, fp32 and bf16 factors."""
import numpy as np
import pytest
import torch

from gpu_util import TOL, dev, to_torch_bf16
from oracle import oracle as O
from segtaco_gb300 import native as N
from segtaco_gb300 import ops, synth

pytestmark = pytest.mark.gpu

CASES = {
    "banded": synth.banded_plus_random(2000, 32, 8, seed=61),
    "powerlaw": synth.power_law(3000, 2500, 1.8, 2000, 0.02, seed=62),
    "short_rows": synth.random_csr(5000, 300, 0.002, seed=63, p_empty=0.3),
}


def _check(A, D, x_dtype, cfg, X32=None, Y32=None):
    X32 = synth.dense(A.M, D, seed=64) if X32 is None else X32
    Y32 = synth.dense(A.K, D, seed=65) if Y32 is None else Y32
    if x_dtype == N.BF16:
        xb, yb = synth.to_bf16_bits(X32), synth.to_bf16_bits(Y32)
        X, Y = to_torch_bf16(xb), to_torch_bf16(yb)
        Xr, Yr = synth.bf16_bits_to_f32(xb), synth.bf16_bits_to_f32(yb)
    else:
        X, Y = torch.from_numpy(X32).cuda(), torch.from_numpy(Y32).cuda()
        Xr, Yr = X32, Y32
    out = torch.full((A.nnz,), float("nan"), device="cuda")
    ops.sddmm(dev(A), X, Y, out, config=cfg)
    torch.cuda.synchronize()
    ref, bound = O.sddmm_f64(A.row_ptr, A.col, A.val, Xr, Yr)
    assert O.max_bound_err(out.cpu().numpy(), ref, bound) <= TOL


@pytest.mark.parametrize("x_dtype", [N.F32, N.BF16])
@pytest.mark.parametrize("kernel,lanes", [(N.SDDMM_AUTO, 0), (N.SDDMM_FIXED, 4),
                                          (N.SDDMM_FIXED, 8), (N.SDDMM_GENERAL, 0)])
@pytest.mark.parametrize("block", [32, 128, 256, 1024])
@pytest.mark.parametrize("name", list(CASES))
def test_sddmm_configs(cuda, name, block, kernel, lanes, x_dtype):
    _check(CASES[name], 64, x_dtype, N.SddmmConfig.make(kernel, block, lanes))


@pytest.mark.parametrize("D", [16, 32, 128, 40])
def test_sddmm_config_widths(cuda, D):
    A = CASES["banded"]
    for lanes in (0, 2, 4, 8, 16):
        _check(A, D, N.F32, N.SddmmConfig.make(N.SDDMM_AUTO, 128, lanes))


def test_sddmm_config_rejects(cuda):
    A = dev(CASES["banded"])
    X = torch.zeros((A.M, 64), device="cuda")
    for bad in (N.SddmmConfig.make(0, 100, 0), N.SddmmConfig.make(0, 8192, 0),
                N.SddmmConfig.make(0, 256, 3), N.SddmmConfig.make(7, 256, 0)):
        with pytest.raises(N.SegtacoError):
            ops.sddmm(A, X, X[:A.K], config=bad)


@pytest.mark.parametrize("x_dtype", [N.F32, N.BF16])
def test_sddmm_autotune_banded_full_size(cuda, x_dtype):
    """The autotuner's configuration on the banded-plus-random SDDMM
    (262,144^2, ~19.1M nonzeros, D = 64), checked on 200,000 sampled nonzeros."""
    A = synth.banded_plus_random(seed=0)
    Ad = dev(A)
    cfg = ops.sddmm_autotune(Ad, 64, x_dtype)
    assert cfg.block_nnz in (32, 64, 128, 256, 512, 1024, 2048, 4096)
    X32, Y32 = synth.dense(A.M, 64, seed=4), synth.dense(A.K, 64, seed=5)
    if x_dtype == N.BF16:
        xb, yb = synth.to_bf16_bits(X32), synth.to_bf16_bits(Y32)
        X, Y = to_torch_bf16(xb), to_torch_bf16(yb)
        Xr, Yr = synth.bf16_bits_to_f32(xb).astype(np.float64), synth.bf16_bits_to_f32(yb).astype(np.float64)
    else:
        X, Y = torch.from_numpy(X32).cuda(), torch.from_numpy(Y32).cuda()
        Xr, Yr = X32.astype(np.float64), Y32.astype(np.float64)
    out = ops.sddmm(Ad, X, Y, config=cfg).cpu().numpy()
    rng = np.random.default_rng(1)
    p = np.sort(rng.choice(A.nnz, 200_000, replace=False))
    rows = np.searchsorted(A.row_ptr, p, side="right") - 1
    a = A.val[p].astype(np.float64)
    exact = a * np.einsum("ij,ij->i", Xr[rows], Yr[A.col[p]])
    bound = np.abs(a) * np.einsum("ij,ij->i", np.abs(Xr[rows]), np.abs(Yr[A.col[p]]))
    assert (np.abs(out[p] - exact) / np.maximum(bound, 1e-30)).max() <= TOL


def test_sddmm_autotune_power_law(cuda):
    A = CASES["powerlaw"]
    cfg = ops.sddmm_autotune(A, 64)
    _check(A, 64, N.F32, cfg)
    cfg = ops.sddmm_autotune(dev(A), 64, N.BF16)
    _check(A, 64, N.BF16, cfg)


@pytest.mark.parametrize("x_dtype", [N.F32, N.BF16])
@pytest.mark.parametrize("name", ["banded", "powerlaw", "short_rows", "rect", "band_3001"])
def test_sddmm_band_kernel(cuda, name, x_dtype):
    """The band kernel (SEGTACO_SDDMM_BAND): in-band dot products from the
    block's dense tile, off-band ones from global memory; banded and unbanded
    patterns, a rectangular A (diagonal at column i * K / M), a last block of
    one row, fp32 and bf16 factors, against the FP64 oracle."""
    A = {"rect": synth.random_csr(3000, 1100, 0.02, seed=66),
         "band_3001": synth.banded_plus_random(3001, 40, 6, seed=67)}.get(name)
    if A is None:
        A = CASES[name]
    _check(A, 64, x_dtype, N.SddmmConfig.make(N.SDDMM_BAND))


def test_sddmm_band_unit_values_and_strides(cuda):
    """vals = NULL (every value 1) and X, Y as strided views (ldx = ldy = 80)."""
    A = CASES["banded"]
    Ad = ops.DeviceCSR.from_host(A, "cuda", with_values=False)
    Xb = torch.from_numpy(synth.dense(A.M, 80, seed=68)).cuda()
    Yb = torch.from_numpy(synth.dense(A.K, 80, seed=69)).cuda()
    X, Y = Xb[:, 8:72], Yb[:, 8:72]
    out = torch.full((A.nnz,), float("nan"), device="cuda")
    ops.sddmm(Ad, X, Y, out, config=N.SddmmConfig.make(N.SDDMM_BAND))
    torch.cuda.synchronize()
    ref, bound = O.sddmm_f64(A.row_ptr, A.col, np.ones_like(A.val), X.cpu().numpy(),
                             Y.cpu().numpy())
    assert O.max_bound_err(out.cpu().numpy(), ref, bound) <= TOL


def test_sddmm_band_autotuned_full_size(cuda):
    """The banded SDDMM configuration at full size through ops.sddmm_autotune
    (band statistics on the device pick the band kernel)."""
    A = synth.banded_plus_random(seed=0)
    Ad = dev(A)
    cfg = ops.sddmm_autotune(Ad, 64)
    assert cfg.kernel == N.SDDMM_BAND
    assert ops.sddmm_autotune(Ad, 64, N.BF16).kernel == N.SDDMM_BAND
    X32, Y32 = synth.dense(A.M, 64, seed=70), synth.dense(A.K, 64, seed=71)
    out = torch.full((A.nnz,), float("nan"), device="cuda")
    ops.sddmm(Ad, torch.from_numpy(X32).cuda(), torch.from_numpy(Y32).cuda(), out, config=cfg)
    torch.cuda.synchronize()
    rows = np.random.default_rng(72).choice(A.M, 2048, replace=False)
    got = out.cpu().numpy()
    for r in rows:
        s0, s1 = int(A.row_ptr[r]), int(A.row_ptr[r + 1])
        ref = A.val[s0:s1].astype(np.float64) * (Y32[A.col[s0:s1]].astype(np.float64) @
                                                  X32[r].astype(np.float64))
        bound = np.abs(A.val[s0:s1]).astype(np.float64) * (
            np.abs(Y32[A.col[s0:s1]]).astype(np.float64) @ np.abs(X32[r]).astype(np.float64))
        assert np.all(np.abs(got[s0:s1] - ref) <= TOL * bound + 1e-30)


@pytest.mark.parametrize("m,k", [(1, 1), (1, 300), (31, 31), (33, 40), (97, 5), (5, 3000)])
def test_sddmm_band_small_shapes(cuda, m, k):
    """Tiny and ragged shapes through the band SDDMM: one row, one column, a
    last block of one row, K smaller than the window, wide rectangles."""
    A = synth.random_csr(m, k, min(1.0, 12.0 / k), seed=m * 11 + k)
    _check(A, 64, N.F32, N.SddmmConfig.make(N.SDDMM_BAND))


def test_sddmm_band_duplicates_and_long_off_band(cuda):
    """Duplicate entries (each its own output) and blocks with more off-band
    nonzeros than the 512-entry list (the rest computed per thread)."""
    rng = np.random.default_rng(78)
    A = synth.random_csr(3000, 3000, 0.02, seed=79)  # ~60 off-band nonzeros per row
    rp, cols, vals = [0], [], []
    for r in range(A.M):
        s0, s1 = int(A.row_ptr[r]), int(A.row_ptr[r + 1])
        c = list(A.col[s0:s1]) + list(A.col[s0:s1:9])
        cols += c
        vals += list(rng.uniform(-1, 1, len(c)).astype(np.float32))
        rp.append(len(cols))
    D = synth.CSR(np.array(rp, np.int32), np.array(cols, np.int32), np.array(vals, np.float32),
                  A.M, A.K)
    _check(D, 64, N.F32, N.SddmmConfig.make(N.SDDMM_BAND))
