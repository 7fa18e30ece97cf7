"""Batched SpMM (segtaco_batch_*): many uneven products in one persistent
launch per kernel variant, direct and through a captured CUDA graph; each
product checked against the FP64 oracle."""
import numpy as np
import pytest
import torch

from gpu_util import TOL, assert_spmm_close, dev, spmm_ref, to_torch_bf16
from oracle import oracle as O
from segtaco_gb300 import native as N
from segtaco_gb300 import ops, synth

pytestmark = pytest.mark.gpu


def make_items(specs):
    items, refs = [], []
    for A, n, bf16 in specs:
        B32 = synth.dense(A.K, n, seed=A.M + n)
        if bf16:
            bits = synth.to_bf16_bits(B32)
            Bd, ref = to_torch_bf16(bits), spmm_ref(A, bits, bf16=True)
        else:
            Bd, ref = torch.from_numpy(B32).cuda(), spmm_ref(A, B32)
        Cd = torch.full((A.M, n), float("nan"), device="cuda")
        items.append((dev(A), Bd, Cd))
        refs.append((A, ref, B32 if not bf16 else bits, bf16))
    return items, refs


def check(items, refs):
    torch.cuda.synchronize()
    for (Ad, Bd, Cd), (A, ref, B, bf16) in zip(items, refs):
        assert_spmm_close(Cd.cpu().numpy(), A, B, bf16=bf16, ref=ref)


def pool_specs(count, seed0=0):
    specs = []
    for m in range(seed0, seed0 + count):
        A, n, _ = synth.pool_matrix(m, min_dim=200, max_dim=6000)
        specs.append((A, n, False))
    return specs


def test_batch_autotuned_pool(cuda):
    specs = pool_specs(24)
    specs.append((synth.power_law(3000, 2500, 1.8, 2000, 0.02, seed=5), 33, False))
    specs.append((synth.random_csr(400, 300, 0.05, seed=6, p_empty=0.2), 8, True))
    specs.append((synth.CSR(np.zeros(4, np.int32), np.zeros(0, np.int32),
                            np.zeros(0, np.float32), 3, 5), 16, False))
    items, refs = make_items(specs)
    b = ops.Batch(items)
    groups, nitems, cfgs = b.info()
    assert groups >= 1 and nitems > 0
    b.run()
    check(items, refs)
    for _, _, Cd in items:
        Cd.fill_(float("nan"))
    for _ in range(2):  # graph captured on the first call, replayed on the second
        b.run(graph=True)
        check(items, refs)
    b.close()


@pytest.mark.parametrize("sched", ["rb_sr", "rb_pr", "eb_sr", "eb_pr"])
def test_batch_explicit_schedules(cuda, sched):
    specs = pool_specs(10, seed0=100)
    items, refs = make_items(specs)
    cfgs = [N.Config.make(schedule=sched) for _ in specs]
    b = ops.Batch(items, configs=cfgs)
    b.run()
    check(items, refs)
    b.close()


def test_batch_matches_single_calls(cuda):
    specs = pool_specs(8, seed0=200)
    items, refs = make_items(specs)
    b = ops.Batch(items)
    _, _, cfgs = b.info()
    b.run()
    torch.cuda.synchronize()
    for (Ad, Bd, Cd), cfg, (A, ref, B, _) in zip(items, cfgs, refs):
        single = ops.spmm(Ad, Bd, config=cfg).cpu().numpy()
        S = ref[1]
        assert np.all(np.abs(Cd.cpu().numpy() - single) <= 2 * TOL * np.maximum(S, 1e-30))


def test_row_stats(cuda):
    A = synth.power_law(5000, 4000, 1.8, 3000, 0.05, seed=9)
    lens = A.row_lengths()
    st = ops.row_stats(dev(A))
    assert st == (int(lens.max()), int((lens == 0).sum()), int((lens >= 32).sum()),
                  int(lens[lens >= 32].sum()))
