"""Serving loop on the GPU: every result checked against the FP64 oracle,
alone and inside a mix of concurrent requests; the device CSR cache under
eviction; device-resident operands; the per-call comparator mode; and the
gated batch run whose bounded wait times out."""
import numpy as np
import pytest
import torch

from gpu_util import TOL, assert_spmm_close, dev, spmm_ref
from oracle import oracle as O
from segtaco_gb300 import native as N
from segtaco_gb300 import ops, synth
from segtaco_gb300.serving import Server

pytestmark = pytest.mark.gpu


def pool(n, seed0=0):
    out = []
    for m in range(seed0, seed0 + n):
        A, nc, _ = synth.pool_matrix(m, min_dim=300, max_dim=8000)
        out.append((A, nc))
    return out


def sddmm_check(A, X, Y, got):
    ref, S = O.sddmm_f64(A.row_ptr, A.col, A.val, X, Y)
    err = np.max(np.abs(got - ref) / np.maximum(S, 1e-30)) if A.nnz else 0.0
    assert err <= TOL, err


def test_server_spmm_sddmm_against_oracle(cuda):
    mats = pool(6)
    with Server(slots=2) as s:
        for i, (A, _) in enumerate(mats):
            s.add_matrix(i, A, pin=True)
        jobs = []
        for i, (A, n) in enumerate(mats):
            B = synth.dense(A.K, n, seed=i)
            Cm = np.full((A.M, n), np.nan, np.float32)
            jobs.append(("spmm", i, B, Cm, s.spmm(i, B, Cm)))
            bits = synth.to_bf16_bits(B)
            Cb = np.full((A.M, n), np.nan, np.float32)
            jobs.append(("bf16", i, bits, Cb, s.spmm(i, bits, Cb)))
            X = synth.dense(A.M, 32, seed=100 + i)
            Y = synth.dense(A.K, 32, seed=200 + i)
            out = np.full(A.nnz, np.nan, np.float32)
            jobs.append(("sddmm", i, (X, Y), out, s.sddmm(i, X, Y, out)))
        for kind, i, B, out, t in jobs:
            assert s.wait(t, 60000) == N.OK
            A = mats[i][0]
            if kind == "sddmm":
                sddmm_check(A, B[0], B[1], out)
            else:
                assert_spmm_close(out, A, B, bf16=(kind == "bf16"))
        st = s.stats()
        assert st["completed"] == len(jobs) and st["failed"] == 0


def test_sddmm_requests_grouped_by_shape(cuda):
    """SDDMM requests of one kernel shape and dtype in a batch share one
    multi-problem launch: 24 requests (D in {16, 32, 64}, fp32 and bf16, four
    matrices) released at once to one slot, every output against FP64."""
    mats = pool(4, seed0=40)
    with Server(slots=1, max_batch=64) as s:
        for i, (A, _) in enumerate(mats):
            s.add_matrix(i, A)
        reqs, keep, checks = [], [], []
        for i, (A, _) in enumerate(mats):
            for D in (16, 32, 64):
                for bf16 in (False, True):
                    X = synth.dense(A.M, D, seed=300 + 10 * i + D)
                    Y = synth.dense(A.K, D, seed=400 + 10 * i + D)
                    if bf16:
                        X, Y = synth.to_bf16_bits(X), synth.to_bf16_bits(Y)
                    out = np.full(A.nnz, np.nan, np.float32)
                    reqs.append(Server.request(N.OP_SDDMM, i, X, out, Y=Y))
                    keep.append((X, Y, out))
                    checks.append((A, X, Y, out, bf16))
        tickets = s.replay(reqs, [0.0] * len(reqs), keep=keep)
        for t in tickets:
            assert s.wait(t, 60000) == N.OK
        for A, X, Y, out, bf16 in checks:
            ref, S = O.sddmm_f64(A.row_ptr, A.col, A.val, X, Y, bf16=bf16)
            if A.nnz:
                assert np.max(np.abs(out - ref) / np.maximum(S, 1e-30)) <= TOL
        st = s.stats()
        assert st["completed"] == len(reqs) and st["failed"] == 0
        assert st["batches"] < len(reqs)  # requests shared batches


def test_same_result_alone_and_in_the_mix(cuda):
    mats = pool(12, seed0=50)
    A0, n0 = mats[0]
    B0 = synth.dense(A0.K, n0, seed=7)
    with Server(slots=3) as s:
        for i, (A, _) in enumerate(mats):
            s.add_matrix(i, A, pin=True)
        alone = np.full((A0.M, n0), np.nan, np.float32)
        assert s.wait(s.spmm(0, B0, alone), 60000) == N.OK
        rng = np.random.default_rng(3)
        keep, reqs, mine = [], [], []
        for k in range(120):
            i = 0 if k % 10 == 5 else int(rng.integers(0, len(mats)))
            A, n = mats[i]
            B = B0 if i == 0 else synth.dense(A.K, n, seed=1000 + k)
            Cm = np.full((A.M, n), np.nan, np.float32)
            keep.append((B, Cm))
            reqs.append(s.request(N.OP_SPMM, i, B, Cm))
            if i == 0:
                mine.append(Cm)
        arrivals = np.cumsum(rng.exponential(50.0, size=len(reqs)))  # 20k requests/s
        tickets = s.replay(reqs, arrivals, keep=keep)
        assert all(s.wait(t, 60000) == N.OK for t in tickets)
        assert s.stats()["mean_batch"] > 1
    ref = spmm_ref(A0, B0)
    for Cm in mine:
        assert_spmm_close(Cm, A0, B0, ref=ref)
        # reduction order is the same; only partition-edge atomics may reorder
        assert np.all(np.abs(Cm - alone) <= 2 * TOL * np.maximum(ref[1], 1e-30))


def test_cache_eviction_keeps_results_right(cuda):
    mats = pool(5, seed0=80)
    def nbytes(A):
        a = lambda n: (n + 255) // 256 * 256
        return a((A.M + 1) * 4) + 2 * a(A.nnz * 4)
    cap = max(nbytes(A) for A, _ in mats) * 2
    with Server(cache_bytes=cap, slots=2) as s:
        for i, (A, _) in enumerate(mats):
            s.add_matrix(i, A, pin=True)
        jobs = []
        for rep in range(3):
            for i, (A, n) in enumerate(mats):
                B = synth.dense(A.K, n, seed=rep * 10 + i)
                Cm = np.full((A.M, n), np.nan, np.float32)
                jobs.append((i, B, Cm, s.spmm(i, B, Cm)))
        for i, B, Cm, t in jobs:
            assert s.wait(t, 60000) == N.OK
            assert_spmm_close(Cm, mats[i][0], B)
        st = s.stats()
        assert st["evictions"] > 0 and st["cache_bytes"] <= cap


def test_device_resident_operands_and_per_call_mode(cuda):
    mats = pool(4, seed0=120)
    for flags in (0, N.SERVER_PER_CALL):
        with Server(flags=flags) as s:
            jobs = []
            for i, (A, n) in enumerate(mats):
                s.add_matrix(i, A)
                B = synth.dense(A.K, n, seed=i)
                Bd = torch.from_numpy(B).cuda()
                Cd = torch.full((A.M, n), float("nan"), device="cuda")
                jobs.append((i, B, Cd, s.spmm(i, Bd, Cd, device=True)))
            for i, B, Cd, t in jobs:
                assert s.wait(t, 60000) == N.OK
                torch.cuda.synchronize()
                assert_spmm_close(Cd.cpu().numpy(), mats[i][0], B)


def test_gated_batch_times_out_and_context_stays_usable(cuda):
    specs = pool(4, seed0=160)
    items, refs = [], []
    for A, n in specs:
        B = synth.dense(A.K, n, seed=A.M)
        items.append((dev(A), torch.from_numpy(B).cuda(),
                      torch.full((A.M, n), float("nan"), device="cuda")))
        refs.append((A, B))
    b = ops.Batch(items)
    N.lib().segtaco_device_status(1)
    gate = torch.zeros(1, dtype=torch.int64, device="cuda")  # nothing ever raises it
    b.run_gated(gate, timeout_s=0.2)
    torch.cuda.synchronize()
    assert N.lib().segtaco_device_status(1) == N.ETIMEOUT
    gate.fill_(len(items))  # everything released: a normal run
    b.run_gated(gate, timeout_s=1.0)
    torch.cuda.synchronize()
    assert N.lib().segtaco_device_status(1) == 0
    for (Ad, Bd, Cd), (A, B) in zip(items, refs):
        assert_spmm_close(Cd.cpu().numpy(), A, B)
    b.close()
