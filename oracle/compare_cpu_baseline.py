"""Times segTACO's CPU product path (Eigen 3.4, oracle/_ref/ref_eigen_time)
beside the timed C port of it (oracle/segtaco_cpu_baseline.c, the bench's
CPU baseline) on the same input and the same threads.

Test infrastructure: runs where the segTACO source tree was present when
oracle/build.py ran (Eigen's sources live only there).

    python oracle/compare_cpu_baseline.py [--frac 0.25] [--threads 0] [--reps 3]

`frac` takes the first rows of the 1M x 1M power-law workload (Zipf 1.8,
N = 128), so that the comparison fits a few tens of seconds.
"""
from __future__ import annotations

import argparse
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from oracle import build as obuild  # noqa: E402
from oracle import oracle as O  # noqa: E402
from segtaco_gb300 import synth  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--frac", type=float, default=0.25)
    ap.add_argument("--threads", type=int, default=0)
    ap.add_argument("--reps", type=int, default=3)
    a = ap.parse_args()
    refs = obuild.build_ref()
    if "ref_eigen_time" not in refs:
        raise SystemExit("segTACO source tree not found: Eigen cannot be built")
    obuild.build_oracle()
    A = synth.power_law(seed=0)
    M = max(1, int(A.M * a.frac))
    rp = np.ascontiguousarray(A.row_ptr[: M + 1])
    nnz = int(rp[M])
    col, val = A.col[:nnz], A.val[:nnz]
    B = synth.dense(A.K, 128, seed=1)
    threads = a.threads if a.threads > 0 else O.cpu_threads()
    with tempfile.TemporaryDirectory() as tmp:
        fin = os.path.join(tmp, "in.bin")
        with open(fin, "wb") as f:
            f.write(np.array([M, A.K, 128, nnz], np.int64).tobytes())
            for x in (rp, col, val, B):
                f.write(np.ascontiguousarray(x).tobytes())
        for th in (threads, 1):
            r = subprocess.run([refs["ref_eigen_time"], fin, str(th), str(a.reps)], check=True,
                               capture_output=True, text=True)
            e = r.stdout.split()
            out = np.empty((M, 128), np.float32)
            O.cpu_spmm(rp, col, val, B, out, th)
            t = []
            for _ in range(a.reps):
                t0 = time.perf_counter()
                O.cpu_spmm(rp, col, val, B, out, th)
                t.append(time.perf_counter() - t0)
            port = statistics.median(t)
            print("rows %d nnz %d threads %d: eigen %.4f s, port %.4f s (port / eigen %.3f); "
                  "checksums %.6e / %.6e" % (M, nnz, th, float(e[1]), port, port / float(e[1]),
                                             float(e[3]), float(out.astype(np.float64).sum())))


if __name__ == "__main__":
    main()
