"""The long-row CTA schedule (segtaco_gb300/csrc/spmm_long.cu), modelled on the
CPU by tests/long_rows_model.py: copies cover exactly what the threads read,
ring slots are reused only after a barrier, the final fold fits in the ring,
and the work list visits every long row and slab once."""
import numpy as np
import pytest

import long_rows_model as LM

C = LM.constants()


def test_constants():
    assert C["kLongCta"] == 128 and C["kLongStage"] % 4 == 0 and C["kLongRing"] >= 2


@pytest.mark.parametrize("esz", [4, 2])
@pytest.mark.parametrize("W", [32, 64, 128])
@pytest.mark.parametrize("pr", [False, True])
@pytest.mark.parametrize("N", [8, 32, 64, 96, 128, 200, 256])
def test_copies_cover_reads(esz, W, pr, N):
    EPC = 16 // esz
    if N % EPC or (W // EPC) > C["kLongCta"]:
        pytest.skip("the planner keeps such widths in the row-block kernel")
    slabs = (N + W - 1) // W
    for slab in range(slabs):
        col0 = slab * W
        for cnt in (1, 17, C["kLongStage"] - 1, C["kLongStage"]):
            done, _ = LM.copies(W, esz, N, col0, cnt, C)
            assert len(done) == len(set(done)), "a chunk copied twice"
            got = set(done)
            for row, colw in LM.reads(W, esz, cnt, pr, C):
                assert row < C["kLongStage"] and colw < W
                if col0 + colw < N:  # columns past N are read but never stored
                    assert (row, colw // EPC) in got, (row, colw)
            # every copy lands inside the stage and inside B's row
            for row, ch in done:
                assert row < cnt and col0 + ch * EPC + EPC <= N


@pytest.mark.parametrize("esz", [4, 2])
@pytest.mark.parametrize("W", [32, 64, 128])
def test_ring_holds_the_fold(esz, W):
    ring_bytes = esz * C["kLongRing"] * C["kLongStage"] * W
    assert 4 * W * 4 <= ring_bytes  # part[4][W] floats of the parallel fold
    smem = ring_bytes + 4 * C["kLongRing"] * C["kLongStage"]
    assert smem <= 227 * 1024


@pytest.mark.parametrize("nst", [1, 2, 3, 4, 5, 8, 33, 200])
def test_pipeline_order(nst):
    assert LM.check_pipeline(nst, C)


def test_pipeline_model_catches_an_early_reuse():
    """The checker itself: a schedule that issues one stage further ahead than
    the ring allows must fail."""
    C2 = dict(C)
    real = LM.pipeline_events

    def too_far(nst, C_):
        ev = real(nst, C_)
        NS = C_["kLongRing"]
        return [("issue", e[1] + 1, (e[1] + 1) % NS) if e[0] == "issue" and e[1] >= NS - 1
                else e for e in ev]
    LM.pipeline_events = too_far
    try:
        with pytest.raises(AssertionError):
            LM.check_pipeline(12, C2)
    finally:
        LM.pipeline_events = real


@pytest.mark.parametrize("seed", range(6))
@pytest.mark.parametrize("T", [1, 7, 512, 2048])
def test_work_list(seed, T):
    rng = np.random.default_rng(seed)
    M = 3000
    lengths = rng.zipf(1.6, M).clip(0, 60_000)
    lengths[rng.random(M) < 0.1] = 0
    nnz = int(lengths.sum())
    front, back, hi_cap, lo_cap = LM.list_rows(lengths, T, nnz)
    assert len(front) <= hi_cap and len(back) <= lo_cap
    for slabs in (1, 2, 5):
        its = LM.items(front, back, hi_cap, slabs)
        seen = [(r, s) for r, s, _ in its]
        want = {(r, s) for r in front + back for s in range(slabs)}
        assert len(seen) == len(set(seen)) and set(seen) == want
        assert all(idx < hi_cap + lo_cap for _, _, idx in its)
        # the longest rows come first
        if front and back:
            assert max(i for i, (r, _, _) in enumerate(its) if r in set(front)) < \
                min(i for i, (r, _, _) in enumerate(its) if r in set(back))
        # the other rows slab by slab (they share one slab of B at a time)
        back_slabs = [s for r, s, _ in its if r in set(back)]
        assert back_slabs == sorted(back_slabs)
