// ref_gpu_timing.cu -- times segTACO's own generic SpMM kernels on this GPU.
//
// REFERENCE-ARM INFRASTRUCTURE ONLY.  Built by baseline/ref_gpu.py against a
// staged copy of segTACO's headers (gpu_library.h and
// matrix_kernels/spmm_{rb,eb}_{sr,pr}.h, unchanged; never committed) into the
// git-ignored baseline/_ref/, and run by bench.py beside this library's own
// kernels.  It calls segTACO's host wrappers exactly as its driver does
// (matrix_experiments/spmm_csr_gpu.h:283-343): each call copies A, B and C to
// the device, times {zero C, kernel} with segTACO's GPUTimer
// (gpu_library.h:818-857), copies C back and frees; the time reported is
// get_gpu_timer_result() (gpu_kernels.cu:20-22), the same figure segTACO's
// sweep logs.
//
// The four dgSPARSE-style generic kernels are the ones that accept any N:
//   spmm_rb_sr  K15 csrspmm_seqreduce_rowbalance_kernel  (spmm_rb_sr.h:187-243)
//   spmm_rb_pr  K20 csrspmm_parreduce_rowbalance_kernel  (spmm_rb_pr.h:223-375)
//   spmm_eb_sr  K24 csrspmm_rowcaching_nnzbalance_kernel (spmm_eb_sr.h:153-423)
//   spmm_eb_pr  K30 csrspmm_parreduce_nnzbalance_kernel  (spmm_eb_pr.h:281-480)
// Their index arithmetic is in bounds for N <= 256 (K15 has no column guard
// past that) with int32 products below 2^31; the caller keeps to that.
//
// Protocol: ref_gpu_timing <in.bin> <out.txt> <warmup> <reps> <name>...
//   in.bin: i64 M, K, N, nnz ; i32 row_ptr[M+1], col[nnz] ; f32 vals[nnz], B[K*N]
//   out.txt: per name one line "name ms_1 ms_2 ... ms_reps checksum" where
//            checksum = sum over C of double(C) after the last call.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "gpu_library.h"
#include "matrix_kernels/spmm_rb_sr.h"
#include "matrix_kernels/spmm_rb_pr.h"
#include "matrix_kernels/spmm_eb_sr.h"
#include "matrix_kernels/spmm_eb_pr.h"

GPUTimer gpu_timer;
float get_gpu_timer_result() { return gpu_timer.get_result(); }

typedef void (*spmm_fn)(taco_tensor_t *, taco_tensor_t *, taco_tensor_t *);

static spmm_fn by_name(const std::string &n) {
  if (n == "spmm_rb_sr") return spmm_rb_sr;
  if (n == "spmm_rb_pr") return spmm_rb_pr;
  if (n == "spmm_eb_sr") return spmm_eb_sr;
  if (n == "spmm_eb_pr") return spmm_eb_pr;
  return nullptr;
}

template <typename T> static std::vector<T> rd(FILE *f, size_t n) {
  std::vector<T> v(n);
  if (n && fread(v.data(), sizeof(T), n, f) != n) {
    fprintf(stderr, "short read\n");
    exit(2);
  }
  return v;
}

int main(int argc, char **argv) {
  if (argc < 6) {
    fprintf(stderr, "usage: ref_gpu_timing in.bin out.txt warmup reps name...\n");
    return 2;
  }
  FILE *fi = fopen(argv[1], "rb");
  if (!fi) return 3;
  auto h = rd<int64_t>(fi, 4);
  const int M = (int)h[0], K = (int)h[1], N = (int)h[2];
  const int64_t nnz = h[3];
  if (N > 256 || (int64_t)M * N >= (1ll << 31) || (int64_t)K * N >= (1ll << 31) ||
      nnz >= (1ll << 31)) {
    fprintf(stderr, "shape outside the generic kernels' int32 / N <= 256 range\n");
    return 4;
  }
  auto pos = rd<int32_t>(fi, M + 1);
  auto crd = rd<int32_t>(fi, nnz);
  auto val = rd<float>(fi, nnz);
  auto Bv = rd<float>(fi, (size_t)K * N);
  fclose(fi);
  std::vector<float> Cv((size_t)M * N, 0.0f);
  // taco_tensor_t views as ds.h:411-458 builds them (CSR A; dense B and C).
  int32_t dimA[2] = {M, K}, dimB[2] = {K, N}, dimC[2] = {M, N};
  int32_t *modeA[2] = {pos.data(), crd.data()};
  int32_t **indA[2] = {nullptr, modeA};
  taco_tensor_t A = {}, B = {}, C = {};
  A.order = 2;
  A.dimensions = dimA;
  A.indices = indA;
  A.vals = val.data();
  B.order = 2;
  B.dimensions = dimB;
  B.vals = Bv.data();
  C.order = 2;
  C.dimensions = dimC;
  C.vals = Cv.data();
  const int warmup = atoi(argv[3]), reps = atoi(argv[4]);
  FILE *fo = fopen(argv[2], "w");
  if (!fo) return 3;
  for (int a = 5; a < argc; ++a) {
    spmm_fn fn = by_name(argv[a]);
    if (!fn) {
      fprintf(stderr, "unknown kernel %s\n", argv[a]);
      return 2;
    }
    for (int i = 0; i < warmup; ++i) fn(&C, &A, &B);
    fprintf(fo, "%s", argv[a]);
    for (int i = 0; i < reps; ++i) {
      fn(&C, &A, &B);
      fprintf(fo, " %.6f", get_gpu_timer_result());
    }
    double sum = 0.0;
    for (size_t i = 0; i < Cv.size(); ++i) sum += (double)Cv[i];
    fprintf(fo, " %.9e\n", sum);
    fflush(fo);
  }
  fclose(fo);
  return 0;
}
