// ref_search.cu -- runs segTACO's own host-callable searches on fixture row_ptr arrays.
//
// TEST INFRASTRUCTURE ONLY (built by oracle/build.py into oracle/_ref/ when the
// segTACO source tree is present; host code only, no GPU is touched).
//
// gpu_library.h is included from the reference tree unchanged; it defines
//   taco_binarySearchAfter  (gpu_library.h:164-184, __device__ __host__)
//   taco_binarySearchBefore (gpu_library.h:185-205, __device__ __host__)
// and the block-start rule of taco_binarySearchBeforeBlock (:206-215), which is
// reproduced here on the host by calling taco_binarySearchBefore for every b.
//
// Protocol: ref_search <in.bin> <out.bin>
//   in  = i64 M, nP ; i32 row_ptr[M+1] ; i32 P[nP] ; i64 nT ; i32 targets[nT]
//   out = for each P: i32 starts[ceil(nnz/P)+1]
//         then i32 before[nT], after[nT]   (over row_ptr[0..M])
#include "gpu_library.h"
#include <vector>

int main(int argc, char **argv) {
  if (argc != 3) return 2;
  FILE *fi = fopen(argv[1], "rb");
  FILE *fo = fopen(argv[2], "wb");
  if (!fi || !fo) return 3;
  int64_t h[2];
  if (fread(h, 8, 2, fi) != 2) return 4;
  int M = (int)h[0];
  std::vector<int> row_ptr(M + 1), P(h[1]);
  if (fread(row_ptr.data(), 4, M + 1, fi) != (size_t)(M + 1)) return 4;
  if (fread(P.data(), 4, h[1], fi) != (size_t)h[1]) return 4;
  int64_t nT;
  if (fread(&nT, 8, 1, fi) != 1) return 4;
  std::vector<int> T(nT);
  if (nT && fread(T.data(), 4, nT, fi) != (size_t)nT) return 4;
  int nnz = row_ptr[M];
  for (int p : P) {
    int nblk = (nnz + p - 1) / p;
    for (int b = 0; b <= nblk; ++b) {
      int s = taco_binarySearchBefore(row_ptr.data(), 0, M, b * p);
      fwrite(&s, 4, 1, fo);
    }
  }
  for (int t : T) {
    int s = taco_binarySearchBefore(row_ptr.data(), 0, M, t);
    fwrite(&s, 4, 1, fo);
  }
  for (int t : T) {
    int s = taco_binarySearchAfter(row_ptr.data(), 0, M, t);
    fwrite(&s, 4, 1, fo);
  }
  fclose(fi);
  fclose(fo);
  return 0;
}
