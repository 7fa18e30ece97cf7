"""Host logic of the serving loop, on the CPU: the server runs with host memory
standing in for the device (no kernels run, outputs are not written), so these
tests check admission, caching, cancellation and failure handling only."""
import threading
import time

import numpy as np
import pytest

from segtaco_gb300 import native as N
from segtaco_gb300 import synth
from segtaco_gb300.serving import Server


def fake(**kw):
    kw.setdefault("flags", N.SERVER_FAKE_DEVICE)
    return Server(**kw)


def mat(seed, M=200, K=150):
    return synth.random_csr(M, K, 0.05, seed=seed)


def bytes_of(A):
    a = lambda n: (n + 255) // 256 * 256
    return a((A.M + 1) * 4) + 2 * a(A.nnz * 4)


def spmm_args(A, n=8):
    return np.zeros((A.K, n), np.float32), np.zeros((A.M, n), np.float32)


def test_requests_complete_and_are_batched():
    A = mat(1)
    with fake(slots=2, fake_delay_us=20000) as s:
        s.add_matrix(7, A)
        tickets = [s.spmm(7, *spmm_args(A)) for _ in range(20)]
        assert all(s.wait(t, 5000) == N.OK for t in tickets)
        st = s.stats()
        assert st["completed"] == 20 and st["failed"] == 0
        assert st["cache_misses"] == 1 and st["cache_hits"] == 19
        # the first request departs alone; the rest arrive while it is in flight
        assert st["batches"] < 20 and st["mean_batch"] > 1
        assert st["p50_us"] > 0 and st["p99_us"] >= st["p50_us"]


def test_add_matrix_rejects_malformed_csr():
    A = mat(2)
    with fake() as s:
        bad = synth.CSR(A.row_ptr.copy(), A.col.copy(), A.val, A.M, A.K)
        bad.col[3] = A.K
        with pytest.raises(N.SegtacoError, match="out of range"):
            s.add_matrix(1, bad)
        bad = synth.CSR(A.row_ptr.copy(), A.col, A.val, A.M, A.K)
        bad.row_ptr[5] = bad.row_ptr[6] + 1
        with pytest.raises(N.SegtacoError, match="decreases"):
            s.add_matrix(1, bad)
        s.add_matrix(1, A)
        with pytest.raises(N.SegtacoError, match="exists"):
            s.add_matrix(1, A)


def test_submit_rejects_unknown_matrix_and_bad_shapes():
    A = mat(3)
    with fake() as s:
        s.add_matrix(1, A)
        B, Cm = spmm_args(A)
        with pytest.raises(N.SegtacoError, match="unknown matrix"):
            s.spmm(99, B, Cm)
        r = s.request(N.OP_SPMM, 1, B, Cm)
        r.N = 0
        with pytest.raises(N.SegtacoError):
            s.submit_request(r, None)
        r = s.request(N.OP_SPMM, 1, B, Cm)
        r.op = 5
        with pytest.raises(N.SegtacoError, match="unknown op"):
            s.submit_request(r, None)


def test_lru_eviction_under_a_small_cache():
    mats = [mat(10 + i) for i in range(3)]
    cap = bytes_of(mats[0]) + bytes_of(mats[1]) + 64
    with fake(cache_bytes=cap, max_batch=1, slots=1) as s:
        for i, A in enumerate(mats):
            s.add_matrix(i, A)
        order = [0, 1, 2, 0, 1, 2]
        ts = [s.spmm(i, *spmm_args(mats[i])) for i in order]
        assert all(s.wait(t, 5000) == N.OK for t in ts)
        st = s.stats()
        assert st["evictions"] >= 3 and st["cache_misses"] == 6
        assert st["cache_bytes"] <= cap


def test_matrix_larger_than_the_cache_fails_alone():
    small, big = mat(20), mat(21, M=2000, K=2000)
    with fake(cache_bytes=bytes_of(small) + 256) as s:
        s.add_matrix(0, small)
        s.add_matrix(1, big)
        t_big = s.spmm(1, *spmm_args(big))
        t_small = s.spmm(0, *spmm_args(small))
        assert s.wait(t_big, 5000) == N.ENOMEM
        assert s.wait(t_small, 5000) == N.OK


def test_staging_cap_exhaustion():
    A = mat(22)
    with fake(staging_bytes=1024) as s:
        s.add_matrix(0, A)
        assert s.wait(s.spmm(0, *spmm_args(A, 64)), 5000) == N.ENOMEM
        st = s.stats()
        assert st["failed"] == 1


def test_injected_allocation_failure_fails_one_request():
    A = mat(23)
    with fake(fail_alloc_at=2, max_batch=1, slots=1) as s:
        s.add_matrix(0, A)
        # allocation 1: the matrix upload; 2: the first request's staging
        ts = [s.spmm(0, *spmm_args(A)) for _ in range(3)]
        assert [s.wait(t, 5000) for t in ts] == [N.ENOMEM, N.OK, N.OK]


def test_cancel_before_admission_only():
    A = mat(24)
    with fake(max_batch=1, slots=1, fake_delay_us=200000) as s:
        s.add_matrix(0, A)
        ts = [s.spmm(0, *spmm_args(A)) for _ in range(3)]
        time.sleep(0.05)  # the first request is admitted and in flight
        assert s.cancel(ts[0]) == N.EBUSY
        assert s.cancel(ts[2]) == N.OK
        assert s.wait(ts[2], 0) == N.ECANCELLED
        assert s.wait(ts[0], 5000) == N.OK and s.wait(ts[1], 5000) == N.OK
        assert s.stats()["cancelled"] == 1


@pytest.mark.filterwarnings("ignore::pytest.PytestUnhandledThreadExceptionWarning")
def test_producer_thread_that_dies():
    A = mat(25)
    got = []

    def producer(s):
        for i in range(5):
            got.append(s.spmm(0, *spmm_args(A)))
        raise RuntimeError("producer dies")

    with fake(fake_delay_us=1000) as s:
        s.add_matrix(0, A)
        th = threading.Thread(target=producer, args=(s,))
        th.start()
        th.join()
        assert len(got) == 5
        assert all(s.wait(t, 5000) == N.OK for t in got)
        s.drain(5000)
        assert s.stats()["pending"] == 0


def test_destroy_with_pending_requests_does_not_hang():
    A = mat(26)
    s = fake(max_batch=1, slots=1, fake_delay_us=100000)
    s.add_matrix(0, A)
    for _ in range(10):
        s.spmm(0, *spmm_args(A))
    t0 = time.time()
    s.close()
    assert time.time() - t0 < 5


def test_many_submitter_threads():
    mats = [mat(30 + i) for i in range(4)]
    with fake(fake_delay_us=500) as s:
        for i, A in enumerate(mats):
            s.add_matrix(i, A)
        tickets = []
        lock = threading.Lock()

        def worker(k):
            for j in range(25):
                i = (k + j) % 4
                t = s.spmm(i, *spmm_args(mats[i]))
                with lock:
                    tickets.append(t)

        ths = [threading.Thread(target=worker, args=(k,)) for k in range(4)]
        for th in ths:
            th.start()
        for th in ths:
            th.join()
        assert len(set(tickets)) == 100
        assert all(s.wait(t, 10000) == N.OK for t in tickets)


def test_replay_open_loop_latency():
    A = mat(40)
    with fake(fake_delay_us=200) as s:
        s.add_matrix(0, A)
        keep = [spmm_args(A) for _ in range(50)]
        reqs = [s.request(N.OP_SPMM, 0, B, Cm) for B, Cm in keep]
        arrivals = np.cumsum(np.full(50, 200.0))  # one request every 200 us
        t0 = time.time()
        tickets = s.replay(reqs, arrivals, keep=keep)
        assert time.time() - t0 >= arrivals[-1] * 1e-6 * 0.9
        assert all(s.wait(t, 5000) == N.OK for t in tickets)
        st = s.stats(reset=True)
        assert st["completed"] == 50 and 0 < st["p50_us"] <= st["p99_us"] <= st["max_us"]
        assert s.stats()["completed"] == 0


def test_sddmm_requests_and_per_call_mode():
    A = mat(41)
    with fake(flags=N.SERVER_FAKE_DEVICE | N.SERVER_PER_CALL, fake_delay_us=100) as s:
        s.add_matrix(0, A)
        X = np.zeros((A.M, 16), np.float32)
        Y = np.zeros((A.K, 16), np.float32)
        out = np.zeros(A.nnz, np.float32)
        ts = [s.sddmm(0, X, Y, out) for _ in range(4)] + [s.spmm(0, *spmm_args(A))]
        assert all(s.wait(t, 5000) == N.OK for t in ts)
        assert s.stats()["batches"] == 5  # one request per batch
