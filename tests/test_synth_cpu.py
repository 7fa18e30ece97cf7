"""The seeded benchmark inputs: sizes and shape properties of each
configuration's matrix, so that a change to a generator shows up here before
it moves a measured number.  Recipes: uniform 16,384^2 with 16 distinct
columns per row; 1M x 1M power law (Zipf row lengths capped at 50,000, 2 %
empty rows, uniform columns) at exponent 1.8 and at 1.922 (the ~10M-nonzero
variant); banded-plus-random 262,144^2 (|i - j| <= 32 plus 8 off-band
columns per row)."""
import numpy as np
import pytest

from segtaco_gb300 import synth


def _check_csr(A):
    rp = A.row_ptr
    assert rp.dtype == np.int32 and A.col.dtype == np.int32 and A.val.dtype == np.float32
    assert rp[0] == 0 and rp[-1] == A.nnz and np.all(np.diff(rp) >= 0)
    assert A.col.min() >= 0 and A.col.max() < A.K
    # columns strictly increasing inside every row (sorted, no duplicates)
    d = np.diff(A.col.astype(np.int64))
    starts = rp[1:-1][(rp[1:-1] > 0) & (rp[1:-1] < A.nnz)]
    inner = np.ones(A.nnz - 1, dtype=bool)
    inner[starts - 1] = False
    assert np.all(d[inner] > 0)
    assert np.all(np.abs(A.val) <= 1.0)


def test_uniform16():
    A = synth.uniform_rows(seed=0)
    assert (A.M, A.K, A.nnz) == (16384, 16384, 262_144)
    assert np.all(A.row_lengths() == 16)
    _check_csr(A)


@pytest.mark.parametrize("zipf_s,nnz", [(1.8, 20_567_850), (1.922, 10_083_633)])
def test_power_law(zipf_s, nnz):
    A = synth.power_law(s=zipf_s, seed=0)
    assert (A.M, A.K, A.nnz) == (1_000_000, 1_000_000, nnz)
    L = A.row_lengths()
    assert L.max() <= 50_000
    assert 0.018 < (L == 0).mean() < 0.022
    _check_csr(A)
    B = synth.power_law(s=zipf_s, seed=0)
    assert np.array_equal(A.col, B.col) and np.array_equal(A.val, B.val)


def test_banded_plus_random():
    A = synth.banded_plus_random(seed=0)
    assert (A.M, A.K, A.nnz) == (262_144, 262_144, 19_135_456)
    _check_csr(A)
    rows = np.repeat(np.arange(A.M), A.row_lengths())
    off = np.abs(A.col.astype(np.int64) - rows) > 32
    assert np.all(np.bincount(rows[off], minlength=A.M) == 8)
