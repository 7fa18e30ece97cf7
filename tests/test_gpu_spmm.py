"""SpMM parity: every schedule against the FP64 oracle (bound-normalised error
<= 1e-5) and against segTACO's Eigen / spmm_cpu_naive outputs (golden
fixtures), through the C ABI."""
import numpy as np
import pytest
import torch

from conftest import golden_cases, load_golden
from gpu_util import TOL, assert_spmm_close, dev, small_cases, spmm_ref, to_torch_bf16
from oracle import oracle as O
from segtaco_gb300 import native as N
from segtaco_gb300 import ops, synth

pytestmark = pytest.mark.gpu
SCHEDULES = ["rb_sr", "rb_pr", "eb_sr", "eb_pr"]
# How a unit is walked and B rows gathered: the planner's choice, the flat
# walk, the row walk, cp.async into a shared-memory ring, or TMA bulk copies.
PATHS = {"auto": 0, "flat": N.FLAG_FLAT_WALK, "rows": N.FLAG_ROW_WALK,
         "ring": N.FLAG_SMEM_RING, "bulk": N.FLAG_SMEM_RING | N.FLAG_TMA_BULK}
SMALL = small_cases()


def run(A, B, cfg=None, **kw):
    Ad = dev(A)
    Bd = torch.from_numpy(np.ascontiguousarray(B)).cuda()
    C = ops.spmm(Ad, Bd, config=cfg, **kw)
    torch.cuda.synchronize()
    return C.cpu().numpy()


@pytest.mark.parametrize("path", list(PATHS))
@pytest.mark.parametrize("sched", SCHEDULES)
@pytest.mark.parametrize("name", golden_cases("spmm_"))
def test_golden(cuda, sched, name, path):
    d = load_golden("spmm_", name)
    A = synth.CSR(d["row_ptr"], d["col"], d["val"], int(d["M"]), int(d["K"]))
    C = run(A, d["B"], N.Config.make(schedule=sched, flags=PATHS[path]))
    r, S = spmm_ref(A, d["B"])
    if r.size:
        assert O.max_bound_err(C, r, S) <= TOL
        # against segTACO's Eigen product: both are within TOL of FP64
        assert O.max_bound_err(C, d["C_eigen"].astype(np.float64), S) <= 2 * TOL


@pytest.mark.parametrize("path", list(PATHS))
@pytest.mark.parametrize("sched", SCHEDULES)
@pytest.mark.parametrize("name", list(SMALL))
def test_small_cases(cuda, sched, name, path):
    A = SMALL[name]
    for n in (1, 4, 8, 33, 64, 128):
        B = synth.dense(A.K, n, seed=n)
        assert_spmm_close(run(A, B, N.Config.make(schedule=sched, flags=PATHS[path])), A, B)


@pytest.mark.parametrize("sched", SCHEDULES)
@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 8, 16, 31, 32, 33, 64, 96, 128, 257])
def test_ragged_widths(cuda, sched, n):
    A = SMALL["powerlaw"]
    B = synth.dense(A.K, n, seed=100 + n)
    assert_spmm_close(run(A, B, N.Config.make(schedule=sched)), A, B)


@pytest.mark.parametrize("sched", SCHEDULES)
def test_tuning_knobs(cuda, sched):
    A = SMALL["powerlaw"]
    B = synth.dense(A.K, 64, seed=5)
    ref = spmm_ref(A, B)
    for col_tile in (4, 16, 32, 64, 128):
        for vec, flags in ((1, 0), (2, 0), (4, 0), (8, 0), (4, N.FLAG_ROW_WALK),
                           (4, N.FLAG_FLAT_WALK), (4, N.FLAG_SMEM_RING)):
            for units in (1, 3, 7, 64, 1024):
                kw = dict(schedule=sched, col_tile=col_tile, vec=vec, flags=flags)
                if sched.startswith("rb"):
                    if units > 8:
                        continue
                    kw["rows_per_unit"] = units
                else:
                    kw["items_per_unit"] = units
                C = run(A, B, N.Config.make(**kw))
                assert_spmm_close(C, A, B, ref=ref)


@pytest.mark.parametrize("sched", SCHEDULES)
def test_bf16_sixteen_column_lanes(cuda, sched):
    """bf16 B with 16 columns per lane (one 32-byte load): G <= 4 groups for
    the parallel schedules; the sequential ones and wider slabs fall back to 8;
    a B only 16-byte aligned or a ragged N to narrower lanes."""
    A = SMALL["powerlaw"]
    for n, tile, off in ((64, 64, 0), (128, 64, 0), (32, 32, 0), (64, 128, 0), (64, 64, 8),
                         (48, 64, 0)):
        B32 = synth.dense(A.K, n + 16, seed=70 + n)
        bits = synth.to_bf16_bits(B32)
        Bb = to_torch_bf16(bits)[:, off:off + n]
        C = ops.spmm(dev(A), Bb, config=N.Config.make(schedule=sched, col_tile=tile, vec=16))
        torch.cuda.synchronize()
        assert_spmm_close(C.cpu().numpy(), A, np.ascontiguousarray(bits[:, off:off + n]),
                          bf16=True)


@pytest.mark.parametrize("sched", SCHEDULES)
def test_l2_hint_flag(cuda, sched):
    A = SMALL["uniform16"]
    B = synth.dense(A.K, 32, seed=6)
    C = run(A, B, N.Config.make(schedule=sched, flags=N.FLAG_L2_HINTS))
    assert_spmm_close(C, A, B)


@pytest.mark.parametrize("path", list(PATHS))
def test_rb_sr_is_the_sequential_fma_order(cuda, path):
    """rb_sr sums each row in storage order with fmaf: bit-exact with the
    sequential FP32 restatement of Eigen's order using fused multiply-adds."""
    for name in ("powerlaw", "uniform16", "one_long_row"):
        A = SMALL[name]
        B = synth.dense(A.K, 32, seed=7)
        C = run(A, B, N.Config.make(schedule="rb_sr", flags=PATHS[path]))
        assert np.array_equal(C, O.spmm_f32_rowseq(A.row_ptr, A.col, A.val, B, fma=True))


@pytest.mark.parametrize("sched", SCHEDULES)
def test_values_default_to_one(cuda, sched):
    A = SMALL["half_empty"]
    B = synth.dense(A.K, 16, seed=8)
    Ad = dev(A, with_values=False)
    C = ops.spmm(Ad, torch.from_numpy(B).cuda(), config=N.Config.make(schedule=sched))
    ones = synth.CSR(A.row_ptr, A.col, np.ones_like(A.val), A.M, A.K)
    assert_spmm_close(C.cpu().numpy(), ones, B)


@pytest.mark.parametrize("sched", SCHEDULES)
def test_strided_and_offset_operands(cuda, sched):
    """Leading dimensions larger than N and 4-byte (not 16-byte) aligned bases."""
    A = SMALL["powerlaw"]
    n = 24
    Bbig = torch.from_numpy(synth.dense(A.K, n + 9, seed=9)).cuda()
    B = Bbig[:, 1:1 + n]  # ldb = n + 9, base offset 4 bytes
    Cbig = torch.full((A.M, n + 3), 7.0, device="cuda")
    C = Cbig[:, 3:]
    ops.spmm(dev(A), B, C_out=C, config=N.Config.make(schedule=sched))
    torch.cuda.synchronize()
    assert_spmm_close(C.cpu().numpy(), A, B.cpu().numpy())
    assert torch.all(Cbig[:, :3] == 7.0)  # columns outside C untouched


@pytest.mark.parametrize("sched", ["rb_pr", "eb_pr"])
@pytest.mark.parametrize("offset", [4, 8])
def test_vec8_alignment(cuda, sched, offset):
    """8-column fp32 lanes load 32 bytes at once: a B whose base is only
    16-byte aligned (offset 4 floats) runs with 4-column lanes, a 32-byte
    aligned one (offset 8) with 8; both give the product."""
    A = SMALL["powerlaw"]
    n = 64
    Bbig = torch.from_numpy(synth.dense(A.K, n + 16, seed=12)).cuda()
    B = Bbig[:, offset:offset + n]  # ldb = n + 16
    C = ops.spmm(dev(A), B, config=N.Config.make(schedule=sched, col_tile=32, vec=8))
    torch.cuda.synchronize()
    assert_spmm_close(C.cpu().numpy(), A, B.cpu().numpy())


@pytest.mark.parametrize("path", list(PATHS))
@pytest.mark.parametrize("sched", SCHEDULES)
def test_bf16_dense_operand(cuda, sched, path):
    """bf16 B with fp32 accumulation: within TOL of the exact product with the
    bf16 values; the error against the fp32 B is the bf16 rounding (stated)."""
    A = SMALL["powerlaw"]
    for n in (8, 64, 128, 3):
        B32 = synth.dense(A.K, n, seed=10 + n)
        bits = synth.to_bf16_bits(B32)
        C = ops.spmm(dev(A), to_torch_bf16(bits),
                     config=N.Config.make(schedule=sched, flags=PATHS[path]))
        torch.cuda.synchronize()
        C = C.cpu().numpy()
        assert_spmm_close(C, A, bits, bf16=True)
        r, S = spmm_ref(A, B32)
        assert O.max_bound_err(C, r, S) <= 2.0 ** -8  # bf16 has 8 significant bits


@pytest.mark.parametrize("sched", SCHEDULES)
def test_workspace_from_caller_and_reuse(cuda, sched):
    A = SMALL["powerlaw"]
    B = torch.from_numpy(synth.dense(A.K, 32, seed=11)).cuda()
    Ad = dev(A)
    cfg = N.Config.make(schedule=sched)
    ws = ops.spmm_workspace_size(Ad, 32, N.F32, cfg)
    buf = torch.empty(max(ws, 256), dtype=torch.uint8, device="cuda")
    C1 = ops.spmm(Ad, B, config=cfg, workspace=buf).clone()
    C2 = ops.spmm(Ad, B, config=cfg, workspace=buf)
    torch.cuda.synchronize()
    assert_spmm_close(C1.cpu().numpy(), A, B.cpu().numpy())
    if sched.endswith("sr") and sched.startswith("rb"):
        assert torch.equal(C1, C2)  # no atomics: bit-identical reruns
    else:
        assert_spmm_close(C2.cpu().numpy(), A, B.cpu().numpy())
    if ws > 256:
        small = torch.empty(ws // 2, dtype=torch.uint8, device="cuda")
        with pytest.raises(N.SegtacoError):
            ops.spmm(Ad, B, config=cfg, workspace=small)


def test_overwrites_c(cuda):
    A = SMALL["half_empty"]
    B = torch.from_numpy(synth.dense(A.K, 16, seed=12)).cuda()
    for sched in SCHEDULES:
        C = torch.full((A.M, 16), float("nan"), device="cuda")
        ops.spmm(dev(A), B, C_out=C, config=N.Config.make(schedule=sched))
        torch.cuda.synchronize()
        assert not torch.isnan(C).any(), sched
        assert_spmm_close(C.cpu().numpy(), A, B.cpu().numpy())


def test_empty_matrix_and_zero_width(cuda):
    A = synth.CSR(np.zeros(6, np.int32), np.zeros(0, np.int32), np.zeros(0, np.float32), 5, 7)
    for sched in SCHEDULES:
        C = run(A, synth.dense(7, 4, seed=1), N.Config.make(schedule=sched))
        assert np.array_equal(C, np.zeros((5, 4), np.float32))
    Ad = dev(SMALL["uniform16"])
    C = ops.spmm(Ad, torch.zeros((Ad.K, 0), device="cuda"))
    assert C.shape == (Ad.M, 0)


@pytest.mark.parametrize("zipf_s", [1.8, 1.922])
def test_full_power_law_all_schedules(cuda, zipf_s):
    """The 1,000,000 x 1,000,000 Zipf workload with N = 128 (exponent 1.8:
    19.9M nonzeros; 1.922: 10.1M): row sums of C against the FP64 product
    A (B 1), and 3000 sampled rows (including the longest ones) against the
    FP64 oracle, for all four schedules."""
    A = synth.power_law(s=zipf_s, seed=0)
    B = synth.dense(A.K, 128, seed=1)
    Ad, Bd = dev(A), torch.from_numpy(B).cuda()
    C = torch.empty((A.M, 128), device="cuda")
    lens = A.row_lengths()
    rng = np.random.default_rng(0)
    rows = np.unique(np.concatenate([np.argsort(lens)[-200:], rng.integers(0, A.M, 2800)]))
    sub_rp = np.concatenate([[0], np.cumsum(lens[rows])]).astype(np.int32)
    sub_col = np.concatenate([A.col[A.row_ptr[r]:A.row_ptr[r + 1]] for r in rows])
    sub_val = np.concatenate([A.val[A.row_ptr[r]:A.row_ptr[r + 1]] for r in rows])
    sub = synth.CSR(sub_rp, sub_col, sub_val, rows.shape[0], A.K)
    ref = spmm_ref(sub, B)
    # linearity: C 1 = A (B 1), in FP64
    b1 = B.astype(np.float64).sum(axis=1)
    b1abs = np.abs(B.astype(np.float64)).sum(axis=1)
    rows_all = np.repeat(np.arange(A.M), lens)
    y = np.bincount(rows_all, weights=A.val.astype(np.float64) * b1[A.col], minlength=A.M)
    yb = np.bincount(rows_all, weights=np.abs(A.val.astype(np.float64)) * b1abs[A.col], minlength=A.M)
    for sched in SCHEDULES:
        for path, flags in PATHS.items():
            C.fill_(float("nan"))
            ops.spmm(Ad, Bd, C_out=C, config=N.Config.make(schedule=sched, flags=flags))
            torch.cuda.synchronize()
            rs = C.double().sum(dim=1).cpu().numpy()
            assert np.all(np.abs(rs - y) <= 2 * TOL * np.maximum(yb, 1e-30)), (sched, path)
            got = C[torch.from_numpy(rows).cuda()].cpu().numpy()
            assert_spmm_close(got, sub, B, ref=ref)


def test_device_status_clean(cuda):
    """No kernel gave up a bounded wait in this session."""
    assert N.lib().segtaco_device_status(1) == N.OK


def test_vendor_comparator_matches_oracle(cuda):
    """segtaco_vendor_spmm (cuSPARSE CSR SpMM, the comparator the spmm_csr_cusparse
    names run) computes the same product within the FP32 bound."""
    A = synth.power_law(3000, 2500, 1.8, 2000, 0.02, seed=21)
    B = synth.dense(A.K, 40, seed=22)
    C = ops.vendor_spmm(dev(A), torch.from_numpy(B).cuda())
    torch.cuda.synchronize()
    assert_spmm_close(C.cpu().numpy(), A, B)
