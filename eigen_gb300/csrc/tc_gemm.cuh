// Tensor-core (tcgen05) trailing update of the low-precision tiers:
//   C (M x N, FP32, column-major) -= A (M x K) * B (K x N)
// A and B are packed first into K-major low-precision buffers (BF16, FP16 or
// TF32, or TF32 split three ways for FP32 accuracy), then a persistent,
// warp-specialized kernel streams them with TMA into a shared-memory ring,
// issues tcgen05.mma from one thread into TMEM accumulators (two buffers, so
// the epilogue of one tile overlaps the MMAs of the next) and applies the
// update C -= acc with coalesced loads/stores.  This is the trailing update
// of PartialPivLU.h:492 and the SYRK of LLT.h:357 for the mixed tiers.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "dense_driver.cuh"

namespace gbs {

enum TcKind {
  TC_BF16 = 0,     // operands rounded to bfloat16 (8-bit significand)
  TC_FP16 = 1,     // operands rounded to float16 (11-bit significand)
  TC_TF32 = 2,     // operands rounded to tf32 (11-bit significand, FP32 range)
  TC_TF32X3 = 3    // FP32 operands split into tf32 hi + lo; a*b ~ hi*hi + hi*lo + lo*hi
};

struct TcWorkspace {
  DevBuf ak, bk;   // packed operands
};

// C -= A * B with A, B FP32 column-major.  lower != 0: only the lower
// triangle of C is updated (SYRK with B = A^T given as b_rs/b_cs strides).
// A(i,k) = A[i*a_rs + k*a_cs], B(k,j) = B[k*b_rs + j*b_cs].
int tc_gemm_sub(cudaStream_t s, int kind, int M, int N, int K, const float* A, int64_t a_rs, int64_t a_cs,
                const float* B, int64_t b_rs, int64_t b_cs, float* C, int64_t ldc, int lower, DeviceStatus* st,
                TcWorkspace& ws, int max_ctas = 0);

}  // namespace gbs
