"""CPU model of the sequential walk's staging and steps (spmm_seq_unit in
segtaco_gb300/csrc/spmm_kernels.cuh): over chunk [y0, y1) the staged ranges
[base, lim) (base a multiple of 4, at most kSeqStage long) and the steps of U
positions from g = p & ~3 take every nonzero exactly once and in order; every
16-byte shared read (index o + 4j .. o + 4j + 3) lies inside the kSeqStage + U
entries of the warp's arrays; staging loads stay inside [base, lim) within
[0, nnz); a step's positions outside [p, end) are never used."""
import re
import os

import numpy as np
import pytest

SRC = os.path.join(os.path.dirname(__file__), "..", "segtaco_gb300", "csrc", "spmm_kernels.cuh")


def constants():
    text = open(SRC).read()
    stage = int(re.search(r"constexpr int kSeqStage = (\d+);", text).group(1))
    m = re.search(r"constexpr int seq_loads\(\) \{ return (\d+); \}", text)
    return stage, int(m.group(1))


def walk(y0, y1, nnz, S, U):
    taken = []
    base, lim = 0, -1
    p = y0
    while p < y1:
        if p >= lim:
            base = p & ~3
            lim = min(base + S, y1)
            assert 0 <= base and lim <= nnz and lim - base <= S
        g = p & ~3
        end = min(g + U, lim)
        o = g - base
        assert o % 4 == 0 and o >= 0
        for j in range(U // 4):
            assert o + 4 * j + 3 < S + U  # one 16-byte shared read inside the arrays
            for k in range(4):
                pos = g + 4 * j + k
                if p <= pos < end:
                    assert pos - base < lim - base  # a staged entry
                    taken.append(pos)
        assert end > p  # progress
        p = end
    return taken


def test_seq_walk_takes_every_nonzero_once():
    S, U = constants()
    assert U % 4 == 0 and S % 4 == 0
    rng = np.random.default_rng(7)
    cases = [(0, 0, 0), (0, 1, 1), (3, 4, 10), (5, 5, 9), (0, S, S), (1, S + 1, S + 7),
             (2, 3 * S + 5, 4 * S)]
    for _ in range(300):
        nnz = int(rng.integers(1, 5 * S))
        y0 = int(rng.integers(0, nnz + 1))
        y1 = int(rng.integers(y0, nnz + 1))
        cases.append((y0, y1, nnz))
    for y0, y1, nnz in cases:
        assert walk(y0, y1, nnz, S, U) == list(range(y0, y1))
