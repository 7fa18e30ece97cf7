"""The slot walk (SEGTACO_FLAG_SLOT_WALK): every slot of a warp walks its own
merge-path chunk.  Products against the FP64 oracle over irregular matrices,
chunk sizes down to one item, the lane shapes it is compiled for, fp32 and
bf16 B, vals = NULL, C overwritten; with one chunk per row range the
sequential schedule is bit-exact with the storage-order FMA chain."""
import numpy as np
import pytest
import torch

from gpu_util import assert_spmm_close, dev, small_cases, to_torch_bf16
from oracle import oracle as O
from segtaco_gb300 import native as N
from segtaco_gb300 import ops, synth

pytestmark = pytest.mark.gpu
CASES = small_cases()


def _cfg(sched, items=0, tile=32, vec=8):
    return N.Config.make(schedule=sched, items_per_unit=items, col_tile=tile, vec=vec,
                         flags=N.FLAG_SLOT_WALK)


def _run(A, Bd, cfg, Cd=None):
    Ad = dev(A)
    assert " walk=3 " in ops.plan_name(Ad, Bd, cfg), ops.plan_name(Ad, Bd, cfg)
    return ops.spmm(Ad, Bd, C_out=Cd, config=cfg)


@pytest.mark.parametrize("items", [1, 3, 16, 64, 512])
@pytest.mark.parametrize("sched", ["eb_pr", "eb_sr"])
@pytest.mark.parametrize("name", list(CASES))
def test_slot_walk_small(cuda, name, sched, items):
    A = CASES[name]
    B = synth.dense(A.K, 64, seed=71)
    Cd = torch.full((A.M, 64), float("nan"), device="cuda")
    _run(A, torch.from_numpy(B).cuda(), _cfg(N.SCHEDULES[sched], items), Cd)
    torch.cuda.synchronize()
    assert_spmm_close(Cd.cpu().numpy(), A, B)


@pytest.mark.parametrize("n,tile,vec", [(32, 32, 8), (64, 32, 8), (40, 32, 8), (128, 32, 8),
                                        (32, 32, 4), (64, 64, 8), (64, 16, 4), (64, 64, 4),
                                        (1, 1, 1), (7, 1, 1)])
def test_slot_walk_shapes(cuda, n, tile, vec):
    A = CASES["powerlaw"]
    B = synth.dense(A.K, n, seed=72)
    C = _run(A, torch.from_numpy(B).cuda(), _cfg(N.EB_PR, 64, tile, vec))
    torch.cuda.synchronize()
    assert_spmm_close(C.cpu().numpy(), A, B)


@pytest.mark.parametrize("vec,tile", [(16, 64), (8, 32), (8, 64)])
def test_slot_walk_bf16(cuda, vec, tile):
    A = CASES["powerlaw"]
    bits = synth.to_bf16_bits(synth.dense(A.K, 128, seed=73))
    C = _run(A, to_torch_bf16(bits), _cfg(N.EB_PR, 64, tile, vec))
    torch.cuda.synchronize()
    assert_spmm_close(C.cpu().numpy(), A, synth.bf16_bits_to_f32(bits))


def test_slot_walk_unit_values(cuda):
    A = CASES["empty_run"]
    B = synth.dense(A.K, 32, seed=74)
    Ad = dev(A, with_values=False)
    Bd = torch.from_numpy(B).cuda()
    cfg = _cfg(N.EB_PR, 16)
    assert " walk=3 " in ops.plan_name(Ad, Bd, cfg)
    C = ops.spmm(Ad, Bd, config=cfg)
    torch.cuda.synchronize()
    ones = synth.CSR(A.row_ptr, A.col, np.ones_like(A.val), A.M, A.K)
    assert_spmm_close(C.cpu().numpy(), ones, B)


def test_slot_walk_eb_sr_one_chunk_bitexact(cuda):
    """One chunk holding the whole matrix: every row one sequential chain."""
    A = synth.power_law(3000, 2500, 1.8, 1500, 0.02, seed=75)
    B = synth.dense(A.K, 32, seed=76)
    want = O.spmm_f32_rowseq(A.row_ptr, A.col, A.val, B, fma=True)
    C = _run(A, torch.from_numpy(B).cuda(), _cfg(N.EB_SR, A.M + A.nnz + 1))
    torch.cuda.synchronize()
    assert np.array_equal(C.cpu().numpy(), want)


@pytest.mark.parametrize("sched", ["eb_pr", "eb_sr"])
def test_slot_walk_full_power_law(cuda, sched):
    """1M x 1M power law (Zipf 1.8), N = 128, checked on 4,096 sampled rows
    and the 16 longest."""
    A = synth.power_law(seed=0)
    B = synth.dense(A.K, 128, seed=1)
    C = _run(A, torch.from_numpy(B).cuda(), _cfg(N.SCHEDULES[sched]))
    torch.cuda.synchronize()
    rng = np.random.default_rng(3)
    rows = np.unique(np.concatenate([rng.choice(A.M, 4096, replace=False),
                                     np.argsort(A.row_lengths())[-16:]]))
    got = C[torch.from_numpy(rows).cuda()].cpu().numpy()
    sub_rp = np.zeros(len(rows) + 1, np.int64)
    np.cumsum(A.row_lengths()[rows], out=sub_rp[1:])
    idx = np.concatenate([np.arange(A.row_ptr[r], A.row_ptr[r + 1]) for r in rows])
    S = synth.CSR(sub_rp.astype(np.int32), A.col[idx], A.val[idx], len(rows), A.K)
    assert_spmm_close(got, S, B)
