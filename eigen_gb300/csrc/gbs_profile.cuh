// Phase profiler and launch counter of libgb300solve.
//
// Every kernel launch of the library is counted (gbs_kernel_launch_count).
// When profiling is enabled (gbs_profile_enable(1)), each phase launch is
// bracketed by CUDA events recorded on the launching stream, tagged with its
// algorithmic flops and bytes; gbs_profile_collect() sums elapsed time per
// phase.  This replaces the reference's BenchTimer-style wall clocks
// (bench/BenchTimer.h) with device-side timing per phase.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace gbs {

enum Phase {
  PH_PANEL = 0,       // LU panel factorization
  PH_LASWP = 1,       // row interchanges
  PH_TRSM_LU = 2,     // A12 <- L11^-1 A12
  PH_GEMM = 3,        // trailing update C -= A B
  PH_POTRF_DIAG = 4,  // Cholesky diagonal block
  PH_TRSM_LLT = 5,    // A21 <- A21 L11^-T
  PH_SYRK = 6,        // trailing update C -= A A^T (lower)
  PH_TRI_SOLVE = 7,   // triangular solves (solve / rcond)
  PH_NORM = 8,        // ||A||_1
  PH_MIXED = 9,       // mixed-precision conversion / refinement kernels
  PH_TC_GEMM = 10,    // tcgen05 tensor-core trailing update
  PH_RESIDUAL = 11,   // FP64 residual r = b - A x
  PH_BATCHED = 12,    // batched small-system kernels
  PH_ROUTER = 13,     // MLP router kernels
  PH_COPY = 14,       // copies / transposes / conversions
  PH_COUNT = 15
};

void count_launch();
bool profiling();
// Records the begin event of a phase launch (no-op when profiling is off).
void prof_begin(cudaStream_t s, int phase);
// Records the end event and tags the launch with its algorithmic work.
void prof_end(cudaStream_t s, int phase, double flops, double bytes);

struct PhaseScope {
  cudaStream_t s;
  int phase;
  double flops, bytes;
  PhaseScope(cudaStream_t s_, int ph, double f, double b) : s(s_), phase(ph), flops(f), bytes(b)
  {
    count_launch();
    prof_begin(s, phase);
  }
  ~PhaseScope() { prof_end(s, phase, flops, bytes); }
};

}  // namespace gbs
