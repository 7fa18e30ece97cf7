// ref_golden.cpp -- runs segTACO's own CPU code on fixture inputs to make golden vectors.
//
// TEST INFRASTRUCTURE ONLY (built by oracle/build.py into oracle/_ref/ when the
// segTACO source tree is present; never shipped, never linked into the product).
//
// The segTACO headers are included from the reference tree unchanged:
//   ds.h                                   to_eigen_csr (:380-397), read_mtx_file (:183-268)
//   matrix_experiments/spmm_csr_gpu.h      spmm_cpu_naive (:110-127)
//   matrix_experiments/sddmm_csr_gpu.h     sddmm_csr_cpu_taco_ref (:9-50)
//   matrix_experiments/spmspv_csr_gpu.h    spmspv_csr_cpu_taco_ref (:9-32)
// and Eigen 3.4.0's sparse x dense product (SparseDenseProduct.h:109-146) is
// reached through EigenCSR * EigenRowMajor exactly as typedef'd at ds.h:32-33.
//
// The experiment headers also define GPU drivers that call the kernel entry
// points; those drivers are never executed here, so the link leaves the kernel
// symbols unresolved (see oracle/build.py) and the SDDMM / SpMSpV GPU names
// that gpu_kernels.cuh comments out get empty stand-ins below.
//
// matrix_experiments/spmspv_csr_gpu.h does not compile against the current
// taco_tensor_t as written (its driver assigns uint8_t*** to int32_t*** at
// :54-58); oracle/build.py compiles a scratch copy in which only those
// allocations are retyped (SPMSPV_CAST_FIX), so spmspv_csr_cpu_taco_ref itself
// is segTACO's code unchanged.
//
// Protocol: ref_golden <mode> <in.bin> <out.bin>, raw little-endian arrays.
//   mode "csr"   : in = i64 M,K,nnz ; i32 rows[nnz], cols[nnz] ; f32 vals[nnz]
//                  out = i32 row_ptr[M+1], col[nnz'] ; f32 vals[nnz']      (to_eigen_csr)
//   mode "spmm"  : in = i64 M,K,N,nnz ; i32 row_ptr[M+1], col[nnz] ; f32 vals[nnz], B[K*N]
//                  out = f32 C_eigen[M*N], C_naive[M*N]
//   mode "spmv"  : in = i64 M,K,nnz ; i32 row_ptr, col ; f32 vals, x[K]    out = f32 y[M]
//   mode "sddmm" : in = i64 M,K,D,nnz ; i32 row_ptr, col ; f64 vals, X[M*D], Y[K*D]
//                  out = f64 out[nnz]
//   mode "spmspv": in = i64 M,K,nnz,nx ; i32 col_ptr[K+1], row_idx[nnz] ; f64 vals[nnz] ;
//                  i32 x_idx[nx] ; f64 x_vals[nx]       out = f64 y[M]
//                  (A as CSC = the CSR of A^T, spmspv_csr_gpu.h:37-43)
//   mode "mtx"   : in = path of a .mtx file (text)                         (read_mtx_file)
//                  out = i64 nrow,ncol,nnz ; i32 indptr[nrow+1], indices[nnz]
#include "ds.h"
#include "timers.h"

void sddmm_csr_gpu_taco(taco_tensor_t *, taco_tensor_t *, taco_tensor_t *, taco_tensor_t *) {}
void sddmm_csr_gpu_warp(taco_tensor_t *, taco_tensor_t *, taco_tensor_t *, taco_tensor_t *) {}
void spmspv_csr_gpu_taco(taco_tensor_t *, taco_tensor_t *, taco_tensor_t *) {}
float get_gpu_timer_result() { return -1.0f; }

#include "matrix_experiments/spmm_csr_gpu.h"
#include "matrix_experiments/sddmm_csr_gpu.h"
#include "matrix_experiments/spmspv_csr_gpu.h"

Timer timer;
std::ofstream log_file;

template <typename T> static std::vector<T> rd(FILE *f, size_t n) {
  std::vector<T> v(n);
  if (n && fread(v.data(), sizeof(T), n, f) != n) {
    fprintf(stderr, "short read\n");
    exit(2);
  }
  return v;
}
template <typename T> static void wr(FILE *f, const T *p, size_t n) {
  if (n && fwrite(p, sizeof(T), n, f) != n) {
    fprintf(stderr, "short write\n");
    exit(2);
  }
}

static taco_tensor_t csr_view(int M, int K, int32_t *pos, int32_t *crd, void *vals) {
  taco_tensor_t t = get_csr_taco_tensor(M, K);  // ds.h:400-409
  t.indices[1][0] = pos;
  t.indices[1][1] = crd;
  t.vals = (float *)vals;
  return t;
}
static taco_tensor_t dense_view(int r, int c, void *vals) {
  taco_tensor_t t;
  t.dimensions = new int32_t[2];
  t.dimensions[0] = r;
  t.dimensions[1] = c;
  t.vals = (float *)vals;
  return t;
}

int main(int argc, char **argv) {
  if (argc != 4) {
    fprintf(stderr, "usage: ref_golden mode in out\n");
    return 2;
  }
  std::string mode = argv[1];
  if (mode == "mtx") {
    int nrow, ncol, nnz;
    std::vector<int> indptr, indices, rowind;
    read_mtx_file(argv[2], nrow, ncol, nnz, indptr, indices, rowind);
    FILE *fo = fopen(argv[3], "wb");
    int64_t h[3] = {nrow, ncol, nnz};
    wr(fo, h, 3);
    wr(fo, indptr.data(), indptr.size());
    wr(fo, indices.data(), indices.size());
    fclose(fo);
    return 0;
  }
  FILE *fi = fopen(argv[2], "rb");
  FILE *fo = fopen(argv[3], "wb");
  if (!fi || !fo) return 3;
  if (mode == "csr") {
    auto h = rd<int64_t>(fi, 3);
    COO coo;
    coo.m = (int)h[0];
    coo.n = (int)h[1];
    coo.nnz = (int)h[2];
    auto r = rd<int32_t>(fi, h[2]);
    auto c = rd<int32_t>(fi, h[2]);
    auto v = rd<float>(fi, h[2]);
    coo.rows = r.data();
    coo.cols = c.data();
    coo.vals = v.data();
    EigenCSR A = to_eigen_csr(coo);
    taco_tensor_t t = to_taco_tensor(A);
    int64_t nnz = t.indices[1][0][coo.m];
    wr(fo, t.indices[1][0], coo.m + 1);
    wr(fo, t.indices[1][1], nnz);
    wr(fo, t.vals, nnz);
  } else if (mode == "spmm") {
    auto h = rd<int64_t>(fi, 4);
    int M = (int)h[0], K = (int)h[1], N = (int)h[2];
    int64_t nnz = h[3];
    auto pos = rd<int32_t>(fi, M + 1);
    auto crd = rd<int32_t>(fi, nnz);
    auto val = rd<float>(fi, nnz);
    auto Bv = rd<float>(fi, (size_t)K * N);
    // Eigen: EigenCSR (ds.h:32) times EigenRowMajor (ds.h:33).
    Eigen::Map<const EigenCSR> A(M, K, nnz, pos.data(), crd.data(), val.data());
    Eigen::Map<const EigenRowMajor> B(Bv.data(), K, N);
    EigenRowMajor C(M, N);
    C.noalias() = A * B;
    wr(fo, C.data(), (size_t)M * N);
    // spmm_cpu_naive accumulates into C: start it at zero.
    std::vector<float> Cn((size_t)M * N, 0.0f);
    taco_tensor_t tA = csr_view(M, K, pos.data(), crd.data(), val.data());
    taco_tensor_t tB = dense_view(K, N, Bv.data());
    taco_tensor_t tC = dense_view(M, N, Cn.data());
    spmm_cpu_naive(&tC, &tA, &tB);
    wr(fo, Cn.data(), Cn.size());
  } else if (mode == "spmv") {
    auto h = rd<int64_t>(fi, 3);
    int M = (int)h[0], K = (int)h[1];
    int64_t nnz = h[2];
    auto pos = rd<int32_t>(fi, M + 1);
    auto crd = rd<int32_t>(fi, nnz);
    auto val = rd<float>(fi, nnz);
    auto xv = rd<float>(fi, K);
    Eigen::Map<const EigenCSR> A(M, K, nnz, pos.data(), crd.data(), val.data());
    Eigen::Map<const EigenVector> x(xv.data(), K);
    EigenVector y(M);
    y.noalias() = A * x;
    wr(fo, y.data(), M);
  } else if (mode == "sddmm") {
    auto h = rd<int64_t>(fi, 4);
    int M = (int)h[0], K = (int)h[1], D = (int)h[2];
    int64_t nnz = h[3];
    auto pos = rd<int32_t>(fi, M + 1);
    auto crd = rd<int32_t>(fi, nnz);
    auto val = rd<double>(fi, nnz);
    auto X = rd<double>(fi, (size_t)M * D);
    auto Y = rd<double>(fi, (size_t)K * D);
    std::vector<double> out(nnz, 0.0);
    // sddmm_csr_cpu_taco_ref(A_out, B_sparse, C, D) reads every operand as double.
    taco_tensor_t tOut = csr_view(M, K, pos.data(), crd.data(), out.data());
    taco_tensor_t tB = csr_view(M, K, pos.data(), crd.data(), val.data());
    taco_tensor_t tC = dense_view(M, D, X.data());
    taco_tensor_t tD = dense_view(K, D, Y.data());
    sddmm_csr_cpu_taco_ref(&tOut, &tB, &tC, &tD);
    wr(fo, out.data(), nnz);
  } else if (mode == "spmspv") {
    auto h = rd<int64_t>(fi, 4);
    int M = (int)h[0], K = (int)h[1], nx = (int)h[3];
    int64_t nnz = h[2];
    auto cptr = rd<int32_t>(fi, K + 1);
    auto ridx = rd<int32_t>(fi, nnz);
    auto val = rd<double>(fi, nnz);
    auto xi = rd<int32_t>(fi, nx);
    auto xv = rd<double>(fi, nx);
    std::vector<double> y(M, -1.0);
    // spmspv_csr_cpu_taco_ref(y, A, x) reads A as CSC (indices[1]: col_ptr,
    // row_idx), x as a sparse vector (indices[0]: pos {0, nx}, crd) and every
    // value array as double.
    taco_tensor_t tA = csr_view(K, M, cptr.data(), ridx.data(), val.data());
    int32_t xpos[2] = {0, nx};
    int32_t *xmode[2] = {xpos, xi.data()};
    int32_t **xind[1] = {xmode};
    taco_tensor_t tx;
    tx.indices = xind;
    tx.vals = (float *)xv.data();
    taco_tensor_t ty = dense_view(M, 1, y.data());
    spmspv_csr_cpu_taco_ref(&ty, &tA, &tx);
    wr(fo, y.data(), M);
  } else {
    fprintf(stderr, "unknown mode\n");
    return 2;
  }
  fclose(fi);
  fclose(fo);
  return 0;
}
