"""A CPU restatement of rb_pr's long-row pieces (segtaco_gb300/csrc/internal.h
piece_layout, spmm_long.cu long_pieces_list_kernel, spmm_kernels.cuh
finish_piece / warp_lower_bound / spmm_piece_unit / spmm_pieces_pass), used by
test_pieces_model_cpu.py to check the index arithmetic without a GPU: where
each piece's (row, first nonzero) pair, counter and partial rows live in the
workspace, which nonzeros each pass over a range of B's rows takes, which
partial rows the last (piece, pass) of a row sums, and the order in which the
work counter hands out (pass, slab, piece) items.

The constants are read from the sources, so the model follows them."""
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "segtaco_gb300", "csrc")


def constants():
    text = open(os.path.join(CSRC, "internal.h")).read()
    out = {}
    for name in ("kPieceLen", "kPieceThreshold", "kPassPieceLen"):
        m = re.search(r"constexpr long long %s = (\d+);" % name, text)
        assert m, name
        out[name] = int(m.group(1))
    m = re.search(r"constexpr int kMaxPieceParts = (\d+);", text)
    assert m
    out["kMaxPieceParts"] = int(m.group(1))
    return out


def layout(nnz, T, S, slabs, W, parts=1):
    """piece_layout: int32 offsets of the pairs, counters and partial rows."""
    multi = 2 * nnz // S + 1
    cap = multi + nnz // T + 1
    ld = slabs * W
    ctr = 2 * cap
    rows = cap if parts > 1 else multi
    part = (ctr + rows * slabs + 63) // 64 * 64
    entries = part + rows * (parts if parts > 1 else 1) * ld
    return dict(multi=multi, cap=cap, ld=ld, ctr=ctr, part=part, entries=entries, rows=rows)


def list_pieces(row_ptr, T, S, L):
    """The list kernel's entries: {entry: (row, first nonzero)} and the rows
    whose counters it clears, in row order (the kernel's atomics give some
    order; every property checked here holds for any)."""
    entries, cleared = {}, []
    n0 = n1 = 0
    for r in range(len(row_ptr) - 1):
        b, ln = row_ptr[r], row_ptr[r + 1] - row_ptr[r]
        if ln < T:
            continue
        n = (ln + S - 1) // S
        if n == 1:
            i = L["multi"] + n1
            n1 += 1
            assert i < L["cap"]
            entries[i] = (r, b)
            cleared.append(i)  # with several passes (all_ctr)
            continue
        i = n0
        n0 += n
        assert i + n <= L["multi"]
        for k in range(n):
            entries[i + k] = (r, b + k * S)
        cleared.append(i)
    return entries, cleared, n0, n1


def warp_lower_bound(col, lo, hi, target):
    """warp_lower_bound: 32 probes per round, the same steps as the device."""
    while hi - lo > 32:
        step = (hi - lo + 31) // 32
        probes = [lo + l * step for l in range(32)]
        ge = [p >= hi or col[p] >= target for p in probes]
        if not any(ge):
            lo += 31 * step + 1
            continue
        f = ge.index(True)
        nhi = lo + f * step
        if f > 0:
            lo = lo + (f - 1) * step + 1
        hi = min(nhi, hi)
    for l in range(32):
        p = lo + l
        if p < hi and col[p] >= target:
            return p
    return hi


def pass_range(col, row_end, y0, S, K, parts, p):
    """[b_p, b_p+1) of the piece starting at y0 (spmm_piece_unit)."""
    y1 = min(y0 + S, row_end)
    if parts == 1:
        return y0, y1
    Kp = (K + parts - 1) // parts
    lo = y0
    for q in range(1, p + 1):
        lo = warp_lower_bound(col, lo, y1, q * Kp)
    hi = warp_lower_bound(col, lo, y1, (p + 1) * Kp) if p + 1 < parts else y1
    return lo, hi


def finish_slots(row_ptr, w, row, y0, S, parts, p, slab, slabs, L):
    """finish_piece: (this piece's partial row or None, counter index, target
    count, the partial rows summed by the last arrival in order)."""
    rs, re_ = row_ptr[row], row_ptr[row + 1]
    n = (re_ - rs + S - 1) // S
    if n == 1 and parts == 1:
        return None, None, None, None
    first = w - (y0 - rs) // S
    slot = w * parts + p
    return slot, first * slabs + slab, n * parts, list(range(first * parts, (first + n) * parts))


def queue_items(total, slabs, parts):
    """spmm_pieces_pass: counter value t -> (pass, slab, list index i)."""
    out = []
    for t in range(total * slabs * parts):
        i = t % total
        ps = t // total
        out.append((ps // slabs, ps % slabs, i))
    return out
