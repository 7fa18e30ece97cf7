"""Seeded random sweep over the SpMM planner's space: random shapes (empty
rows, long rows, ragged N), fp32 and bf16 B at random offsets, and random
combinations of schedule, slab width, lane width, unit size, depth and walk,
each against the FP64 oracle (bound-normalised error <= 1e-5).  Combinations
the planner rejects must fail with a status, not run.  The same random shapes
drive SDDMM (random D, fp32 / bf16 factors at offsets) and SpMV / SpMSpV."""
import numpy as np
import pytest
import torch

from gpu_util import TOL, assert_spmm_close, dev, to_torch_bf16
from oracle import oracle as O
from segtaco_gb300 import native as N
from segtaco_gb300 import ops, synth

pytestmark = pytest.mark.gpu
CASES = 160


def random_matrix(rng):
    kind = rng.integers(0, 4)
    M = int(rng.integers(1, 2500))
    K = int(rng.integers(1, 2500))
    seed = int(rng.integers(0, 1 << 30))
    if kind == 0:
        return synth.random_csr(M, K, float(rng.uniform(0, 0.02)), seed=seed,
                                p_empty=float(rng.uniform(0, 0.6)))
    if kind == 1:
        rows = {int(r): int(rng.integers(1, 4 * K + 1)) for r in rng.integers(0, M, 3)}
        return synth.random_csr(M, K, float(rng.uniform(0, 0.005)), seed=seed, long_rows=rows)
    if kind == 2:
        return synth.power_law(M, K, 1.8, max(1, K), 0.05, seed=seed)
    return synth.uniform_rows(M, max(K, 16), int(rng.integers(1, 16)), seed=seed)


@pytest.mark.parametrize("case", range(CASES))
def test_random_config(cuda, case):
    rng = np.random.default_rng(1000 + case)
    A = random_matrix(rng)
    n = int(rng.choice([1, 2, 3, 4, 7, 8, 16, 31, 32, 33, 64, 96, 128, 200]))
    bf16 = bool(rng.integers(0, 2))
    off = int(rng.choice([0, 1, 4, 8]))
    B32 = synth.dense(A.K, n + 16, seed=case)
    kw = dict(schedule=str(rng.choice(["rb_sr", "rb_pr", "eb_sr", "eb_pr"])),
              col_tile=int(rng.choice([0, 4, 8, 16, 32, 64, 128, 256])),
              vec=int(rng.choice([0, 1, 2, 4, 8] + ([16] if bf16 else []))),
              items_per_unit=int(rng.choice([0, 1, 7, 64, 512, 4096])),
              rows_per_unit=int(rng.choice([0, 1, 3, 8])),
              depth=int(rng.choice([0, 4, 8])),
              flags=int(rng.choice([0, N.FLAG_ROW_WALK, N.FLAG_FLAT_WALK, N.FLAG_L2_HINTS])))
    cfg = N.Config.make(**kw)
    if bf16:
        bits = synth.to_bf16_bits(B32)
        Bd = to_torch_bf16(bits)[:, off:off + n]
        Bref = np.ascontiguousarray(bits[:, off:off + n])
    else:
        Bd = torch.from_numpy(B32).cuda()[:, off:off + n]
        Bref = np.ascontiguousarray(B32[:, off:off + n])
    C = torch.full((A.M, n), float("nan"), device="cuda")
    try:
        ops.spmm(dev(A), Bd, C_out=C, config=cfg)
    except N.SegtacoError as e:
        # the planner's refusals: a status, never a launch
        assert e.code in (N.EINVAL, N.EUNSUPPORTED), (kw, e)
        return
    torch.cuda.synchronize()
    assert_spmm_close(C.cpu().numpy(), A, Bref, bf16=bf16)


@pytest.mark.parametrize("case", range(60))
def test_random_sddmm(cuda, case):
    rng = np.random.default_rng(5000 + case)
    A = random_matrix(rng)
    D = int(rng.choice([1, 3, 4, 8, 16, 24, 32, 64, 96, 128, 256, 300]))
    bf16 = bool(rng.integers(0, 2))
    off = int(rng.choice([0, 1, 4, 8, 16]))
    X = synth.dense(A.M, D + 32, seed=case)
    Y = synth.dense(A.K, D + 32, seed=case + 1)
    if bf16:
        X, Y = synth.to_bf16_bits(X), synth.to_bf16_bits(Y)
        Xd, Yd = to_torch_bf16(X)[:, off:off + D], to_torch_bf16(Y)[:, off:off + D]
    else:
        Xd = torch.from_numpy(X).cuda()[:, off:off + D]
        Yd = torch.from_numpy(Y).cuda()[:, off:off + D]
    out = torch.full((A.nnz,), float("nan"), device="cuda")
    ops.sddmm(dev(A), Xd, Yd, out)
    ref, bound = O.sddmm_f64(A.row_ptr, A.col, A.val, np.ascontiguousarray(X[:, off:off + D]),
                             np.ascontiguousarray(Y[:, off:off + D]), bf16=bf16)
    if ref.size:
        assert O.max_bound_err(out.cpu().numpy(), ref, bound) <= TOL


@pytest.mark.parametrize("case", range(40))
def test_random_spmv_spmspv(cuda, case):
    rng = np.random.default_rng(7000 + case)
    A = random_matrix(rng)
    x = synth.dense(A.K, 1, seed=case).reshape(-1)
    y = torch.full((A.M,), float("nan"), device="cuda")
    ops.spmv(dev(A), torch.from_numpy(x).cuda(), y)
    S = O.spmm_absbound(A.row_ptr, A.col, A.val, x.reshape(-1, 1)).reshape(-1)
    assert O.max_bound_err(y.cpu().numpy(), O.spmv_f64(A.row_ptr, A.col, A.val, x), S) <= TOL
    At = A.transpose()
    nx = int(rng.integers(0, A.K + 1))
    idx = np.sort(rng.permutation(A.K)[:nx]).astype(np.int32)
    xv = rng.uniform(-1, 1, nx).astype(np.float32)
    ys = ops.spmspv(dev(At), torch.from_numpy(idx).cuda(), torch.from_numpy(xv).cuda(), A.M)
    ref, bound = O.spmspv_f64(At.row_ptr, At.col, At.val, A.M, idx, xv)
    assert O.max_bound_err(ys.cpu().numpy(), ref, bound) <= TOL


@pytest.mark.parametrize("case", range(20))
def test_random_batch(cuda, case):
    """A batch of 3-16 random problems, each with its own random config and
    dtype (so several kernel-variant groups), run directly and through the
    captured graph."""
    rng = np.random.default_rng(9000 + case)
    items, refs, cfgs = [], [], []
    for m in range(int(rng.integers(3, 17))):
        A = random_matrix(rng)
        n = int(rng.choice([1, 4, 8, 16, 33, 64, 128]))
        bf16 = bool(rng.integers(0, 2))
        B32 = synth.dense(A.K, n, seed=100 * case + m)
        if bf16:
            bits = synth.to_bf16_bits(B32)
            Bd, Bref = to_torch_bf16(bits), bits
        else:
            Bd, Bref = torch.from_numpy(B32).cuda(), B32
        Cd = torch.full((A.M, n), float("nan"), device="cuda")
        items.append((dev(A), Bd, Cd))
        refs.append((A, Bref, bf16))
        cfgs.append(N.Config.make(
            schedule=str(rng.choice(["rb_sr", "rb_pr", "eb_sr", "eb_pr"])),
            col_tile=int(rng.choice([0, 16, 32, 64, 128])),
            vec=int(rng.choice([0, 1, 2, 4, 8] + ([16] if bf16 else []))),
            items_per_unit=int(rng.choice([0, 7, 64, 512])),
            rows_per_unit=int(rng.choice([0, 1, 3, 8]))))
    try:
        b = ops.Batch(items, configs=cfgs)
    except N.SegtacoError as e:
        assert e.code in (N.EINVAL, N.EUNSUPPORTED), e
        return
    for graph in (False, True, True):
        for _, _, Cd in items:
            Cd.fill_(float("nan"))
        b.run(graph=graph)
        torch.cuda.synchronize()
        for (_, _, Cd), (A, Bref, bf16) in zip(items, refs):
            assert_spmm_close(Cd.cpu().numpy(), A, Bref, bf16=bf16)
    b.close()
