"""Seeded synthetic CSR workloads (numpy PCG64).

segTACO's sweep reads SuiteSparse matrices (new_names.txt) that are not
available here; these generators stand in for them with the shapes, sizes and
value distributions of the benchmark workloads:

* ``uniform_rows``      16384 x 16384, exactly 16 distinct uniform columns per row
* ``power_law``         1,000,000 x 1,000,000, Zipf(1.8) row lengths capped at
                        50,000, 2 % empty rows, uniform columns
* ``banded_plus_random`` 262,144 x 262,144, band |i-j| <= 32 plus 8 uniform
                        off-band columns per row
* ``pool_matrix``       one matrix of the uneven batched/served pool
                        (log-uniform size, lognormal row lengths, one of four
                        structures, N in {16, 32, 64, 128})

Values are uniform in [-1, 1] as float32.  Columns inside a row are sorted and
distinct, which is the CSR that ds.h:380-397 (to_eigen_csr) builds.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

POOL_SEED_BASE = 0x5E67AC0


@dataclasses.dataclass
class CSR:
    row_ptr: np.ndarray  # int32 [M+1]
    col: np.ndarray      # int32 [nnz]
    val: np.ndarray      # float32 [nnz]
    M: int
    K: int

    @property
    def nnz(self) -> int:
        return int(self.row_ptr[self.M])

    def row_lengths(self) -> np.ndarray:
        return np.diff(self.row_ptr)

    def transpose(self) -> "CSR":
        """CSR of A^T (i.e. the CSC of A), stable in row order."""
        rows = np.repeat(np.arange(self.M, dtype=np.int32), self.row_lengths())
        order = np.argsort(self.col, kind="stable")
        t_col = rows[order].astype(np.int32)
        t_val = self.val[order]
        counts = np.bincount(self.col, minlength=self.K)
        t_ptr = np.zeros(self.K + 1, np.int64)
        np.cumsum(counts, out=t_ptr[1:])
        return CSR(t_ptr.astype(np.int32), t_col, t_val, self.K, self.M)


def _sorted_unique(keys: np.ndarray) -> np.ndarray:
    """Sorted distinct values (sort + adjacent difference; faster than np.unique)."""
    k = np.sort(keys)
    if k.shape[0] == 0:
        return k
    keep = np.empty(k.shape[0], bool)
    keep[0] = True
    np.not_equal(k[1:], k[:-1], out=keep[1:])
    return k[keep]


def _from_keys(keys: np.ndarray, M: int, K: int, rng) -> CSR:
    """Sorted distinct int64 keys row*K+col -> CSR with U[-1,1] values."""
    rows = (keys // K).astype(np.int64)
    col = (keys % K).astype(np.int32)
    counts = np.bincount(rows, minlength=M)
    row_ptr = np.zeros(M + 1, np.int64)
    np.cumsum(counts, out=row_ptr[1:])
    if row_ptr[-1] >= 2 ** 31:
        raise ValueError("nnz does not fit int32 indices")
    val = rng.uniform(-1.0, 1.0, size=col.shape[0]).astype(np.float32)
    return CSR(row_ptr.astype(np.int32), col, val, M, K)


def dense(rows: int, cols: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return rng.uniform(-1.0, 1.0, size=(rows, cols)).astype(np.float32)


def to_bf16_bits(a: np.ndarray) -> np.ndarray:
    """float32 -> bf16 bit patterns (uint16), round to nearest even."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u >> 16) & 1) + 0x7FFF
    return ((u + r) >> 16).astype(np.uint16)


def bf16_bits_to_f32(h: np.ndarray) -> np.ndarray:
    return (np.ascontiguousarray(h, dtype=np.uint16).astype(np.uint32) << 16).view(np.float32)


def uniform_rows(M: int = 16384, K: int = 16384, per_row: int = 16, seed: int = 0) -> CSR:
    """Exactly `per_row` distinct uniform columns per row (no replacement)."""
    rng = np.random.default_rng(seed)
    cols = rng.integers(0, K, size=(M, per_row), dtype=np.int64)
    cols.sort(axis=1)
    while True:
        bad = np.nonzero((np.diff(cols, axis=1) == 0).any(axis=1))[0]
        if bad.size == 0:
            break
        redo = rng.integers(0, K, size=(bad.size, per_row), dtype=np.int64)
        redo.sort(axis=1)
        cols[bad] = redo
    keys = (np.arange(M, dtype=np.int64)[:, None] * K + cols).reshape(-1)
    return _from_keys(keys, M, K, rng)


def zipf_lengths(rng, n: int, s: float, cap: int) -> np.ndarray:
    """n draws of L with P(L = l) proportional to l**-s on 1..cap."""
    w = np.arange(1, cap + 1, dtype=np.float64) ** (-s)
    cdf = np.cumsum(w)
    cdf /= cdf[-1]
    u = rng.random(n)
    return (np.searchsorted(cdf, u, side="right") + 1).astype(np.int64)


def _rows_with_uniform_cols(rng, lengths: np.ndarray, K: int) -> np.ndarray:
    """Keys row*K+col, `lengths[i]` uniform draws per row, deduplicated, sorted."""
    M = lengths.shape[0]
    rows = np.repeat(np.arange(M, dtype=np.int64), lengths)
    cols = rng.integers(0, K, size=rows.shape[0], dtype=np.int64)
    return _sorted_unique(rows * K + cols)


def power_law(M: int = 1_000_000, K: int = 1_000_000, s: float = 1.8, cap: int = 50_000,
              p_empty: float = 0.02, seed: int = 0) -> CSR:
    rng = np.random.default_rng(seed)
    lengths = zipf_lengths(rng, M, s, min(cap, K))
    lengths[rng.random(M) < p_empty] = 0
    keys = _rows_with_uniform_cols(rng, lengths, K)
    return _from_keys(keys, M, K, rng)


def banded_plus_random(M: int = 262_144, half_band: int = 32, extra: int = 8,
                       seed: int = 0) -> CSR:
    """|i-j| <= half_band, plus `extra` distinct uniform off-band columns per row."""
    rng = np.random.default_rng(seed)
    K = M
    i = np.arange(M, dtype=np.int64)
    off = np.arange(-half_band, half_band + 1, dtype=np.int64)
    band = i[:, None] + off[None, :]
    band_keys = (i[:, None] * K + band)[(band >= 0) & (band < K)]
    cols = rng.integers(0, K, size=(M, extra), dtype=np.int64)
    todo = np.arange(M)
    # Redraw every row whose draws hit the band or repeat a column.
    while True:
        sub = cols[todo]
        cs = np.sort(sub, axis=1)
        bad = (np.abs(sub - i[todo, None]) <= half_band).any(axis=1) | \
            (np.diff(cs, axis=1) == 0).any(axis=1)
        todo = todo[bad]
        if todo.size == 0:
            break
        cols[todo] = rng.integers(0, K, size=(todo.size, extra), dtype=np.int64)
    extra_keys = (i[:, None] * K + cols).reshape(-1)
    keys = np.sort(np.concatenate([band_keys, extra_keys]))
    return _from_keys(keys, M, K, rng)


STRUCTURES = ("uniform", "banded", "blockdiag", "zipf")
POOL_NS = (16, 32, 64, 128)


def pool_matrix(m: int, min_dim: int = 1000, max_dim: int = 200_000):
    """Matrix m of the uneven pool: returns (CSR, N, structure)."""
    rng = np.random.default_rng(POOL_SEED_BASE + m)
    M = int(math.floor(math.exp(rng.uniform(math.log(min_dim), math.log(max_dim)))))
    K = M
    structure = STRUCTURES[int(rng.integers(0, 4))]
    N = POOL_NS[int(rng.integers(0, 4))]
    mu = math.log(12.0) - 0.5
    if structure == "zipf":
        lengths = zipf_lengths(rng, M, 1.8, K)
    else:
        lengths = np.rint(rng.lognormal(mu, 1.0, size=M)).astype(np.int64)
        lengths = np.clip(lengths, 0, K)
    if structure == "uniform" or structure == "zipf":
        keys = _rows_with_uniform_cols(rng, lengths, K)
    elif structure == "banded":
        rows = np.repeat(np.arange(M, dtype=np.int64), lengths)
        start = np.repeat(np.arange(M, dtype=np.int64) - lengths // 2, lengths)
        offs = np.arange(rows.shape[0], dtype=np.int64) - np.repeat(
            np.cumsum(lengths) - lengths, lengths)
        cols = start + offs
        ok = (cols >= 0) & (cols < K)
        keys = _sorted_unique(rows[ok] * K + cols[ok])
    else:  # block-diagonal 64 x 64 blocks, up to L distinct columns inside the row's block
        lengths = np.minimum(lengths, 64)
        rows = np.repeat(np.arange(M, dtype=np.int64), lengths)
        base = (rows // 64) * 64
        width = np.minimum(64, K - base)
        cols = base + rng.integers(0, 1 << 30, size=rows.shape[0]) % width
        keys = _sorted_unique(rows * K + cols)
    return _from_keys(keys, M, K, rng), N, structure


def random_csr(M: int, K: int, density: float, seed: int, p_empty: float = 0.0,
               long_rows: dict | None = None) -> CSR:
    """Small irregular test matrices: Bernoulli(density) pattern, optional empty
    rows and rows forced to a given length (long_rows = {row: length})."""
    rng = np.random.default_rng(seed)
    lengths = rng.binomial(K, density, size=M).astype(np.int64)
    if p_empty:
        lengths[rng.random(M) < p_empty] = 0
    if long_rows:
        for r, L in long_rows.items():
            lengths[r] = min(L, K)
    keys = []
    for r in range(M):
        L = int(lengths[r])
        if L:
            c = rng.choice(K, size=L, replace=False)
            keys.append(r * K + np.sort(c).astype(np.int64))
    keys = np.concatenate(keys) if keys else np.zeros(0, np.int64)
    return _from_keys(np.sort(keys), M, K, rng)


def csr_from_dense_pattern(pattern: np.ndarray, vals: np.ndarray | None = None) -> CSR:
    M, K = pattern.shape
    r, c = np.nonzero(pattern)
    row_ptr = np.zeros(M + 1, np.int32)
    np.cumsum(np.bincount(r, minlength=M), out=row_ptr[1:])
    v = (vals[r, c] if vals is not None else np.ones(r.shape[0])).astype(np.float32)
    return CSR(row_ptr, c.astype(np.int32), v, M, K)
