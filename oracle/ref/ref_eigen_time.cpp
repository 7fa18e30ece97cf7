// ref_eigen_time.cpp -- times segTACO's CPU product path (Eigen 3.4,
// EigenCSR * EigenRowMajor as typedef'd at ds.h:32-33) on one input.
//
// TEST INFRASTRUCTURE ONLY (built by oracle/build.py into oracle/_ref/ where the
// segTACO source tree is present).  oracle/compare_cpu_baseline.py runs it
// beside the timed C port (segtaco_cpu_baseline.c) on the same input and
// threads, to show that the port times what Eigen's product takes.
//
// Protocol: ref_eigen_time <in.bin> <threads> <reps>
//   in.bin: i64 M, K, N, nnz ; i32 row_ptr[M+1], col[nnz] ; f32 vals[nnz], B[K*N]
//   prints: "eigen <median seconds> <threads> <checksum>"
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <vector>

#include "ds.h"

template <typename T> static std::vector<T> rd(FILE *f, size_t n) {
  std::vector<T> v(n);
  if (n && fread(v.data(), sizeof(T), n, f) != n) {
    fprintf(stderr, "short read\n");
    exit(2);
  }
  return v;
}

int main(int argc, char **argv) {
  if (argc != 4) return 2;
  FILE *fi = fopen(argv[1], "rb");
  if (!fi) return 3;
  auto h = rd<int64_t>(fi, 4);
  const int M = (int)h[0], K = (int)h[1], N = (int)h[2];
  const int64_t nnz = h[3];
  auto pos = rd<int32_t>(fi, M + 1);
  auto crd = rd<int32_t>(fi, nnz);
  auto val = rd<float>(fi, nnz);
  auto Bv = rd<float>(fi, (size_t)K * N);
  fclose(fi);
  const int threads = atoi(argv[2]), reps = atoi(argv[3]);
  Eigen::setNbThreads(threads);
  Eigen::Map<const EigenCSR> A(M, K, nnz, pos.data(), crd.data(), val.data());
  Eigen::Map<const EigenRowMajor> B(Bv.data(), K, N);
  EigenRowMajor C(M, N);
  C.noalias() = A * B;  // warm-up (page-in, thread pool)
  std::vector<double> t;
  for (int r = 0; r < reps; ++r) {
    auto t0 = std::chrono::steady_clock::now();
    C.noalias() = A * B;
    auto t1 = std::chrono::steady_clock::now();
    t.push_back(std::chrono::duration<double>(t1 - t0).count());
  }
  std::sort(t.begin(), t.end());
  double sum = 0.0;
  for (int64_t i = 0; i < (int64_t)M * N; ++i) sum += C.data()[i];
  printf("eigen %.6f %d %.9e\n", t[t.size() / 2], Eigen::nbThreads(), sum);
  return 0;
}
