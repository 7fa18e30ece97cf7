"""CPU checks of rb_pr's long-row pieces through the restatement in
pieces_model.py: the warp-wide bisection, the passes' ranges (every nonzero of
a long row in exactly one (piece, pass), sorted rows or not), the workspace
offsets of pairs, counters and partial rows, and the work counter's order."""
import bisect

import numpy as np
import pytest

import pieces_model as PM


def test_constants():
    c = PM.constants()
    assert c["kPieceThreshold"] <= c["kPassPieceLen"] <= c["kPieceLen"]
    assert c["kMaxPieceParts"] >= 2


@pytest.mark.parametrize("n", [0, 1, 5, 31, 32, 33, 64, 100, 1023, 1024, 4096, 50_000])
def test_lower_bound_matches_bisect_on_sorted(n):
    rng = np.random.default_rng(n)
    col = np.sort(rng.integers(0, max(1, 3 * n), n)).tolist()  # duplicates included
    for target in [-1, 0] + rng.integers(0, 3 * n + 2, 20).tolist() + [10**9]:
        for lo, hi in ((0, n), (n // 3, n), (0, n // 2)):
            got = PM.warp_lower_bound(col, lo, hi, target)
            want = bisect.bisect_left(col, target, lo, hi)
            assert got == want, (n, lo, hi, target)


@pytest.mark.parametrize("seed", range(6))
def test_lower_bound_stays_in_range_on_unsorted(seed):
    rng = np.random.default_rng(100 + seed)
    n = int(rng.integers(1, 5000))
    col = rng.integers(0, 1000, n).tolist()
    for _ in range(50):
        lo = int(rng.integers(0, n))
        hi = int(rng.integers(lo, n + 1))
        got = PM.warp_lower_bound(col, lo, hi, int(rng.integers(-5, 1005)))
        assert lo <= got <= hi


def _csr(rng, M, K, lengths, sort):
    rows, cols = [], []
    for r, ln in enumerate(lengths):
        c = rng.choice(K, size=min(ln, K), replace=False) if ln else np.zeros(0, np.int64)
        if sort:
            c = np.sort(c)
        cols.append(c)
    row_ptr = np.zeros(M + 1, np.int64)
    np.cumsum([len(c) for c in cols], out=row_ptr[1:])
    return row_ptr.tolist(), np.concatenate(cols).astype(np.int64).tolist()


@pytest.mark.parametrize("parts,sort,S", [(1, True, 4096), (2, True, 2048), (3, True, 2048),
                                          (8, True, 512), (2, False, 2048), (5, False, 1024)])
def test_passes_cover_every_nonzero_once(parts, sort, S):
    rng = np.random.default_rng(parts * 10 + sort)
    K, T = 10_007, 512
    lengths = rng.binomial(40, 0.5, 400).tolist()
    lengths[3], lengths[50], lengths[51], lengths[399] = 9000, 512, 511, 2 * S
    lengths[200] = S + 1
    M = len(lengths)
    row_ptr, col = _csr(rng, M, K, lengths, sort)
    nnz = row_ptr[-1]
    slabs, W = 4, 32
    L = PM.layout(nnz, T, S, slabs, W, parts)
    entries, cleared, n0, n1 = PM.list_pieces(row_ptr, T, S, L)
    seen = {}
    slots = set()
    for w, (row, y0) in entries.items():
        for p in range(parts):
            b, e = PM.pass_range(col, row_ptr[row + 1], y0, S, K, parts, p)
            assert y0 <= b <= e <= min(y0 + S, row_ptr[row + 1])
            for q in range(b, e):
                assert q not in seen, (row, q)
                seen[q] = (w, p)
                if sort and parts > 1:  # a pass gathers only from its range of B's rows
                    Kp = (K + parts - 1) // parts
                    assert p * Kp <= col[q] < (p + 1) * Kp
            for slab in range(slabs):
                slot, ci, target, summed = PM.finish_slots(row_ptr, w, row, y0, S, parts, p, slab,
                                                           slabs, L)
                if slot is None:
                    assert parts == 1 and lengths[row] <= S
                    continue
                assert 0 <= slot < L["rows"] * parts
                assert (L["part"] + (slot + 1) * L["ld"]) <= L["entries"]
                assert L["ctr"] + ci < L["part"]  # counters below the partial rows
                first = ci // slabs
                assert first in cleared  # its counter was cleared by the list pass
                assert slot in summed and len(summed) == target
                slots.add((slot, slab))
    long_nz = sum(row_ptr[r + 1] - row_ptr[r] for r in range(M) if lengths[r] >= T)
    assert len(seen) == long_nz
    # every (piece, pass) of every slab has its own partial row
    assert len(slots) == sum(1 for _ in entries) * parts * slabs or parts == 1


@pytest.mark.parametrize("total,slabs,parts", [(1, 1, 1), (7, 4, 2), (100, 3, 8), (5, 1, 3)])
def test_queue_order(total, slabs, parts):
    items = PM.queue_items(total, slabs, parts)
    assert len(items) == len(set(items)) == total * slabs * parts
    assert items == sorted(items)  # pass-major, then slab, then piece
