// FP64-accurate residual R = B - A X on the bf16 tensor cores (Ozaki scheme;
// see ozaki.cu).  A is sliced once (OzakiMatrix::prepare); each residual
// slices X and runs one tcgen05 product kernel.
#pragma once

#include <cuda.h>

#include "dense_driver.cuh"

namespace gbs {

// A's digit slices: 8 bf16 matrices, row-scaled, K-major (8 x mp x ldk), the
// row exponents and row maxima (non-finite rows make their residuals NaN),
// and the tensor map of the stacked slices.  16 n^2 bytes.
struct OzakiMatrix {
  DevBuf slices, rowmax, row_exp;
  CUtensorMap tmA;
  int n = 0, mp = 0;
  int64_t ldk = 0;
  bool ready = false;
  // A general, column-major (symmetric matrices are passed as full copies).
  int prepare(cudaStream_t s, int n, const double* A, int64_t lda);
};

struct OzakiWork {
  DevBuf xs, colmax, col_exp, part;
};

// R = B - A X (B null: R = A X) for nrhs <= 16 columns; err: the timeout flag
// the product kernel's bounded waits set.
int ozaki_residual(cudaStream_t s, OzakiMatrix& M, int nrhs, const double* X, int64_t ldx, const double* B,
                   int64_t ldb, double* R, int64_t ldr, OzakiWork& w, int* err);

}  // namespace gbs
