// Batched split-BF16 GEMM on the 5th-generation tensor cores (tcgen05, TMEM accumulators).
#pragma once
#include <cuda_bf16.h>

#include "lmw_internal.h"

namespace lmw {

// One CTA computes one problem: D[128 x nseg*n] (FP32, row-major, leading dimension ldd) where column block s is
//   sum over the split terms of A_t[:, kseg[s]:kseg[s+1]] * B_t[:, kseg[s]:kseg[s+1]]^T
// with A (128 rows) and B (n rows) stored K-major in BF16 (row stride lda / ldb elements, 16-byte aligned rows).
// The further split pieces of A and B sit at a + p * a_ps and b + p * b_ps. Terms: 1 = hi*hi; 3 = lo*hi + hi*lo +
// hi*hi; 6 (three-piece split hi, mid, lo) = every product down to 2^-24.
struct GemmProblem {
  const __nv_bfloat16 *a;
  const __nv_bfloat16 *b;
  float *d;
  long a_ps, b_ps;  // element stride between split pieces
  int lda, ldb, ldd;
  int arows;    // rows of A that hold data (1..128); the others are zero and their D rows are not written
  int n;        // multiple of 16, 16..256
  int nseg;     // 1..3
  int kseg[4];  // multiples of 16; kseg[0] = 0
};

// Launch on `stream`: one CTA per problem. `err` (device int) receives a nonzero code if a wait on the tensor
// cores ran out (the CTA then releases its tensor memory and returns).
void tc_gemm_launch(const GemmProblem *probs_dev, int nprob, int terms, int *err, cudaStream_t stream, int layout_variant = 0);
// Split FP32 values into BF16 pieces: out[0..n) = hi, out[lo..lo+n) = lo (and out[2lo..] = lo2 when pieces = 3).
void split_bf16_launch(const float *in, __nv_bfloat16 *out, long n, long lo, int pieces, cudaStream_t stream);

// One problem from host arrays (A 128 x K, B N x K, D 128 x N, FP32), for validating the kernel. Returns the
// kernel's error code (0 when every wait completed).
int tc_gemm_selftest(const float *A, const float *B, float *D, int N, int K, int terms, int variant);

}  // namespace lmw
