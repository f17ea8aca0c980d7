/*
 * libgb300solve -- GB300 (sm_103a) dense factor-and-solve behind a C ABI.
 *
 * Drop-in boundary for Eigen's dense factor-and-solve path (Eigen 3.3.90):
 * plain pointers and sizes, column-major storage with a leading dimension,
 * no C++ or torch types.  Three layers, each mirroring an existing reference
 * interface:
 *
 *   1. Plug-in level -- the two functions Eigen's LAPACKE backend replaces
 *      (Eigen/src/Cholesky/LLT_LAPACKE.h:42-93,
 *       Eigen/src/LU/PartialPivLU_LAPACKE.h:42-77).  Same return values as
 *      llt_inplace<>::blocked (LLT.h:331-360) and
 *      partial_lu_impl<>::blocked_lu (PartialPivLU.h:426-496).
 *   2. LAPACK level -- same semantics as the reference's own LAPACK shim
 *      (lapack/lu.cpp:14-89, lapack/cholesky.cpp:14-72): 1-based ipiv,
 *      info < 0 for a bad argument, info = k+1 for the first zero pivot /
 *      failing column.  Bad arguments are reported through info only.
 *   3. Decomposition objects -- device-resident factors mirroring
 *      Eigen::LLT / Eigen::PartialPivLU (compute, info, solve, rcond,
 *      matrixLLT / matrixLU, permutationP, determinant), with host-buffer and
 *      device-buffer variants.
 *
 * All entry points return a gbs_status.  There is no CPU fallback: if no
 * usable sm_103a device is present every call returns GBS_NO_DEVICE.
 * Objects are not thread-safe; distinct objects may be used from distinct host
 * threads concurrently (each owns its stream and workspace).
 *
 * Stream ordering of the device-buffer variants (*_compute_device,
 * *_solve_device): the work runs on the object's stream.  By default that is a
 * blocking stream of its own, which waits for work queued earlier on the
 * legacy default stream; data produced on any other stream must be made ready
 * by the caller first, or the object bound to the producing stream with
 * gbs_*_set_stream.
 */
#ifndef GB300SOLVE_H
#define GB300SOLVE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum gbs_status {
  GBS_SUCCESS = 0,
  GBS_NUMERICAL_ISSUE = 1,    /* Eigen::NumericalIssue (Constants.h:434-444) */
  GBS_INVALID_ARGUMENT = 2,   /* Eigen::InvalidInput */
  GBS_NO_CONVERGENCE = 3,     /* Eigen::NoConvergence: refinement stalled */
  GBS_CUDA_ERROR = 4,
  GBS_NO_DEVICE = 5,
  GBS_TIMEOUT = 6,            /* an inter-CTA wait ran out of time; context stays usable */
  GBS_NOT_INITIALIZED = 7,
  GBS_OUT_OF_MEMORY = 8
} gbs_status;

typedef enum gbs_dtype { GBS_F64 = 0, GBS_F32 = 1 } gbs_dtype;
typedef enum gbs_uplo { GBS_LOWER = 0, GBS_UPPER = 1 } gbs_uplo;

/* Last error text of the calling thread (never NULL). */
const char* gbs_last_error(void);
/* Library version string. */
const char* gbs_version(void);
/* Number of usable sm_103a devices (0 when none). */
int gbs_device_count(void);

/* Failure detection (no counterpart in the reference, whose CPU code has no
 * inter-thread waits).  Every wait of one CTA on another (grid barriers of the
 * cooperative panel kernels, ready flags of the persistent triangular solve,
 * mbarrier waits of the tensor-core GEMM) gives up after a wall-time limit;
 * the launch then ends, the call returns GBS_TIMEOUT (-(100 + GBS_TIMEOUT)
 * where a call returns statuses negated) and the CUDA context stays usable.
 * gbs_set_wait_limit sets that limit for the launches issued after it, process
 * wide; seconds <= 0 restores the 2 s default.  Returns the previous limit in
 * seconds. */
double gbs_set_wait_limit(double seconds);
/* Diagnostics of the bounded waits: each runs one launch whose wait can never
 * be satisfied and reports what the caller would see, on a private stream.
 *  - gbs_selftest_solve_timeout: the persistent triangular solve of an n x n
 *    system with the first block's ready flag never published;
 *  - gbs_selftest_barrier_timeout: a grid barrier that counts one CTA more than
 *    the launch has.
 * Both return GBS_TIMEOUT when the waits expired and the launch ended cleanly
 * (any other status is a failure of the mechanism). */
int gbs_selftest_solve_timeout(int n);
int gbs_selftest_barrier_timeout(void);

/* ------------------------------------------------------------------ 1. plug-in
 * Replaces internal::llt_inplace<Scalar,Lower|Upper>::blocked(m)
 * (Eigen/src/Cholesky/LLT.h:331-360; LAPACKE form LLT_LAPACKE.h:64-88).
 * a: host, column-major n x n, lda >= n; the lower (upper) triangle is read
 * and overwritten by L (U = L^T); the other triangle is left untouched.
 * Returns -1 on success, else the 0-based first column whose pivot is not
 * positive (the matrix is then left as the reference leaves it: columns before
 * that block factored, later blocks untouched).  A negative status below -1 is
 * -(100 + gbs_status) on a library error. */
int64_t gbs_llt_blocked_d(int64_t n, double* a, int64_t lda, int upper);
int64_t gbs_llt_blocked_s(int64_t n, float* a, int64_t lda, int upper);

/* Replaces internal::partial_lu_impl<Scalar,ColMajor,int>::blocked_lu
 * (Eigen/src/LU/PartialPivLU.h:426-496; LAPACKE form PartialPivLU_LAPACKE.h:47-71).
 * a: host, column-major rows x cols, lda >= rows.  Writes 0-based row
 * transpositions (min(rows,cols) of them) and the number of actual swaps.
 * Returns the first exactly-zero pivot or -1; below -1 as above. */
int64_t gbs_partial_lu_blocked_d(int64_t rows, int64_t cols, double* a, int64_t lda,
                                 int* row_transpositions, int* nb_transpositions);
int64_t gbs_partial_lu_blocked_s(int64_t rows, int64_t cols, float* a, int64_t lda,
                                 int* row_transpositions, int* nb_transpositions);

/* ------------------------------------------------------------------ 2. LAPACK
 * Same arguments and results as the reference's shim, lapack/lu.cpp:14-41
 * (getrf) and :46-89 (getrs, trans = 'N'|'T'|'C'), lapack/cholesky.cpp:14-36
 * (potrf, uplo = 'L'|'U') and :41-72 (potrs).  Host buffers. */
int gbs_dgetrf(const int* m, const int* n, double* a, const int* lda, int* ipiv, int* info);
int gbs_sgetrf(const int* m, const int* n, float* a, const int* lda, int* ipiv, int* info);
int gbs_dgetrs(const char* trans, const int* n, const int* nrhs, const double* a, const int* lda,
               const int* ipiv, double* b, const int* ldb, int* info);
int gbs_sgetrs(const char* trans, const int* n, const int* nrhs, const float* a, const int* lda,
               const int* ipiv, float* b, const int* ldb, int* info);
int gbs_dpotrf(const char* uplo, const int* n, double* a, const int* lda, int* info);
int gbs_spotrf(const char* uplo, const int* n, float* a, const int* lda, int* info);
int gbs_dpotrs(const char* uplo, const int* n, const int* nrhs, const double* a, const int* lda,
               double* b, const int* ldb, int* info);
int gbs_spotrs(const char* uplo, const int* n, const int* nrhs, const float* a, const int* lda,
               float* b, const int* ldb, int* info);

/* Allocation-free LU.  This entry point has no counterpart in the reference.
 *
 * For callers that must not let a library allocate device memory: a real-time
 * control loop that runs under a no-allocation rule (the GPU analogue of the
 * reference's EIGEN_RUNTIME_NO_MALLOC mode), or an application that hands all
 * device memory to its own pool and a fixed budget.  cudaMalloc can block,
 * can synchronize the device and can fail when memory is short, so such a
 * caller cannot use gbs_dgetrf, which allocates its workspace on demand.
 *
 * Same factorization and results as gbs_dgetrf (1-based ipiv, LAPACK info),
 * but on DEVICE buffers, stream-ordered on `stream` (a cudaStream_t; NULL is
 * the legacy default stream), and without calling cudaMalloc, cudaFree or any
 * allocating routine.  The scratch it needs (256 KiB: the panel's
 * candidate-exchange buffers and a status word) is a fixed array inside the
 * library, which every GPU that loads the library holds until the process
 * exits.
 *   d_a     device, column-major m x n, lda >= max(1, m); overwritten by L\U
 *   d_ipiv  device, min(m, n) ints; receives 1-based pivot rows
 *   d_info  device, one int; receives 0, or k+1 for the first exactly-zero
 *           pivot k, or -106 if an inter-CTA wait timed out
 * Returns GBS_SUCCESS once the work is enqueued, GBS_INVALID_ARGUMENT for bad
 * arguments or for m or n above 65536 (the limit of the fixed scratch).
 * All calls share the one scratch array, which keeps the last call's contents
 * (each call resets what must start at zero): calls whose work overlaps on the
 * GPU (different streams, or several host threads) race on it and must be
 * serialized by the caller.  The first call on a device does the set-up for
 * that device: it loads every kernel that a call of any shape can launch (CUDA
 * otherwise loads kernels lazily, on first launch, which can take device
 * memory) and looks up the array's device address.  Make that first call
 * before any section that must not allocate; later calls of any shape then
 * allocate nothing.  Profiling
 * (gbs_profile_enable) must stay off, since it creates CUDA events. */
int gbs_dgetrf_noalloc(int m, int n, double* d_a, int lda, int* d_ipiv, int* d_info, void* stream);

/* ------------------------------------------------------------------ 3. objects
 * gbs_llt mirrors Eigen::LLT<Matrix<S,Dynamic,Dynamic>, UpLo> (LLT.h:56-230):
 *   compute   LLT::compute (LLT.h:424-452): copy, ||A||_1 (symmetric, stored
 *             triangle read), blocked factorization, info.
 *   info      LLT::info(): GBS_SUCCESS or GBS_NUMERICAL_ISSUE.
 *   solve     LLT::solve / _solve_impl (LLT.h:477-505).
 *   rcond     LLT::rcond (LLT.h:161-166, ConditionEstimator.h:157-169).
 *   matrix    LLT::matrixLLT (LLT.h:172-176).
 * Scalars are double for GBS_F64 objects and float for GBS_F32 objects. */
typedef struct gbs_llt gbs_llt;
int gbs_llt_create(gbs_llt** out, int dtype, int uplo);
int gbs_llt_destroy(gbs_llt* llt);
int gbs_llt_compute(gbs_llt* llt, int64_t n, const void* a, int64_t lda);            /* host A */
int gbs_llt_compute_device(gbs_llt* llt, int64_t n, const void* d_a, int64_t lda);   /* device A, not modified */
int gbs_llt_info(const gbs_llt* llt);
int64_t gbs_llt_failed_column(const gbs_llt* llt);  /* -1 when info() is Success */
int gbs_llt_solve(gbs_llt* llt, int64_t nrhs, const void* b, int64_t ldb, void* x, int64_t ldx);
int gbs_llt_solve_device(gbs_llt* llt, int64_t nrhs, const void* d_b, int64_t ldb, void* d_x, int64_t ldx);
int gbs_llt_rcond(gbs_llt* llt, double* rcond);
int gbs_llt_l1_norm(const gbs_llt* llt, double* l1);
int gbs_llt_matrix(gbs_llt* llt, void* out, int64_t ld);   /* whole n x n working matrix (matrixLLT) */
void* gbs_llt_device_matrix(gbs_llt* llt, int64_t* ld);     /* device pointer of the factor */
int gbs_llt_synchronize(gbs_llt* llt);
/* Use a caller-owned CUDA stream (cudaStream_t) instead of the object's own. */
int gbs_llt_set_stream(gbs_llt* llt, void* stream);
/* LLT::rankUpdate(v, sigma) (LLT.h:461-472, llt_rank_update_lower LLT.h:231-299):
 * the factor of A + sigma v v^T from the factor of A, by Givens rotations
 * (sigma > 0) or the downdate (sigma <= 0).  info() becomes
 * GBS_NUMERICAL_ISSUE when a downdate would lose definiteness (the factor is
 * then updated up to that column, as the reference leaves it), else
 * GBS_SUCCESS; l1_norm() keeps the value of compute(), as in the reference.
 * v: n scalars, host (rank_update) or device (rank_update_device). */
int gbs_llt_rank_update(gbs_llt* llt, const void* v, double sigma);
int gbs_llt_rank_update_device(gbs_llt* llt, const void* d_v, double sigma);

/* gbs_lu mirrors Eigen::PartialPivLU<Matrix<S,Dynamic,Dynamic>> (PartialPivLU.h:75-311):
 *   compute        PartialPivLU::compute (PartialPivLU.h:514-536)
 *   matrix         matrixLU()
 *   permutation    permutationP().indices() (PermutationMatrix.h:82-88)
 *   transpositions the 0-based row transpositions (m_rowsTranspositions)
 *   solve          _solve_impl (PartialPivLU.h:224-244); transpose != 0 gives
 *                  _solve_impl_transposed (PartialPivLU.h:246-271), i.e. A^T x = b
 *   rcond          PartialPivLU::rcond (PartialPivLU.h:184-188)
 *   determinant    PartialPivLU::determinant (PartialPivLU.h:539-543) */
typedef struct gbs_lu gbs_lu;
int gbs_lu_create(gbs_lu** out, int dtype);
int gbs_lu_destroy(gbs_lu* lu);
int gbs_lu_compute(gbs_lu* lu, int64_t n, const void* a, int64_t lda);
int gbs_lu_compute_device(gbs_lu* lu, int64_t n, const void* d_a, int64_t lda);
int64_t gbs_lu_first_zero_pivot(const gbs_lu* lu);   /* -1 when none */
int gbs_lu_nb_transpositions(const gbs_lu* lu);
int gbs_lu_solve(gbs_lu* lu, int64_t nrhs, const void* b, int64_t ldb, void* x, int64_t ldx, int transpose);
int gbs_lu_solve_device(gbs_lu* lu, int64_t nrhs, const void* d_b, int64_t ldb, void* d_x, int64_t ldx,
                        int transpose);
int gbs_lu_rcond(gbs_lu* lu, double* rcond);
int gbs_lu_l1_norm(const gbs_lu* lu, double* l1);
int gbs_lu_determinant(gbs_lu* lu, double* det);
/* A^-1 = solve(I), PartialPivLU::inverse() (PartialPivLU.h:197-201): n x n,
 * column-major, to host x (ld ldx) or device d_x (stream-ordered). */
int gbs_lu_inverse(gbs_lu* lu, void* x, int64_t ldx);
int gbs_lu_inverse_device(gbs_lu* lu, void* d_x, int64_t ldx);
int gbs_lu_matrix(gbs_lu* lu, void* out, int64_t ld);
int gbs_lu_transpositions(gbs_lu* lu, int* out);
int gbs_lu_permutation(gbs_lu* lu, int* out);
void* gbs_lu_device_matrix(gbs_lu* lu, int64_t* ld);
int gbs_lu_synchronize(gbs_lu* lu);
int gbs_lu_set_stream(gbs_lu* lu, void* stream);

/* gbs_ldlt mirrors Eigen::LDLT<Matrix<S,Dynamic,Dynamic>, UpLo> (LDLT.h:59-287),
 * Cholesky with diagonal pivoting, A = P^T L D L^T P:
 *   compute        LDLT::compute (LDLT.h:491-524): copy, ||A||_1 (symmetric,
 *                  stored triangle read), ldlt_inplace<UpLo>::unblocked
 *                  (LDLT.h:291-383); the transpositions are the reference's,
 *                  bit for bit
 *   info           GBS_SUCCESS or GBS_NUMERICAL_ISSUE, the reference's rule: a
 *                  zero pivot whose column is not zero below the diagonal, or
 *                  a nonzero pivot after a zero one
 *   sign           LDLT.h:22 SignMatrix: 0 PositiveSemiDef, 1 NegativeSemiDef,
 *                  2 ZeroSign, 3 Indefinite; is_positive / is_negative as
 *                  isPositive() / isNegative() (LDLT.h:169-181)
 *   solve          _solve_impl (LDLT.h:540-577), with D's pseudo-inverse
 *   rcond          LDLT::rcond (ConditionEstimator.h:157-169)
 *   matrix         matrixLDLT(): L strictly below (above, Upper) the diagonal,
 *                  D on it, the other triangle as given
 *   vector_d       vectorD(); transpositions: transpositionsP().indices() */
typedef struct gbs_ldlt gbs_ldlt;
int gbs_ldlt_create(gbs_ldlt** out, int dtype, int uplo);
int gbs_ldlt_destroy(gbs_ldlt* ldlt);
int gbs_ldlt_compute(gbs_ldlt* ldlt, int64_t n, const void* a, int64_t lda);
int gbs_ldlt_compute_device(gbs_ldlt* ldlt, int64_t n, const void* d_a, int64_t lda);
int gbs_ldlt_info(const gbs_ldlt* ldlt);
int gbs_ldlt_sign(const gbs_ldlt* ldlt);
int gbs_ldlt_is_positive(const gbs_ldlt* ldlt);
int gbs_ldlt_is_negative(const gbs_ldlt* ldlt);
int gbs_ldlt_solve(gbs_ldlt* ldlt, int64_t nrhs, const void* b, int64_t ldb, void* x, int64_t ldx);
int gbs_ldlt_solve_device(gbs_ldlt* ldlt, int64_t nrhs, const void* d_b, int64_t ldb, void* d_x, int64_t ldx);
int gbs_ldlt_rcond(gbs_ldlt* ldlt, double* rcond);
int gbs_ldlt_l1_norm(const gbs_ldlt* ldlt, double* l1);
int gbs_ldlt_matrix(gbs_ldlt* ldlt, void* out, int64_t ld);
int gbs_ldlt_vector_d(gbs_ldlt* ldlt, void* out);
int gbs_ldlt_transpositions(gbs_ldlt* ldlt, int* out);
void* gbs_ldlt_device_matrix(gbs_ldlt* ldlt, int64_t* ld);
int gbs_ldlt_synchronize(gbs_ldlt* ldlt);
int gbs_ldlt_set_stream(gbs_ldlt* ldlt, void* stream);

/* ------------------------------------------------------------------ BLAS level 3
 * The reference's BLAS shim on the GPU, same arguments and results as
 * blas/level3_impl.h: ?gemm_ (:12-75), ?trsm_ (:77-176), ?syrk_ (:357-433).
 *   gemm   C = alpha op(A) op(B) + beta C (op: 'N', 'T' or 'C'); beta = 0 sets
 *          C to zero without reading it; k = 0 only scales C
 *   trsm   solves op(A) X = B (side 'L') or X op(A) = B (side 'R') for the
 *          uplo triangle of A, then X *= alpha; with diag 'U' the diagonal is
 *          not read; X overwrites B
 *   syrk   C = alpha op(A) op(A)^T + beta C (op 'N': A n x k; 'T'/'C': A k x n)
 *          on the uplo triangle of C only
 * Returns 0, or the position of the first invalid argument (the number the
 * reference reports through xerbla; the text is in gbs_last_error()), or
 * -(100 + gbs_status) on a library error.  Host variants copy their operands
 * to the GPU and C (B for trsm) back; *_device variants take device buffers
 * and run stream-ordered on `stream` (NULL: the legacy default stream). */
int gbs_dgemm(const char* transa, const char* transb, const int* m, const int* n, const int* k, const double* alpha,
              const double* a, const int* lda, const double* b, const int* ldb, const double* beta, double* c,
              const int* ldc);
int gbs_sgemm(const char* transa, const char* transb, const int* m, const int* n, const int* k, const float* alpha,
              const float* a, const int* lda, const float* b, const int* ldb, const float* beta, float* c,
              const int* ldc);
int gbs_dgemm_device(const char* transa, const char* transb, const int* m, const int* n, const int* k,
                     const double* alpha, const double* d_a, const int* lda, const double* d_b, const int* ldb,
                     const double* beta, double* d_c, const int* ldc, void* stream);
int gbs_sgemm_device(const char* transa, const char* transb, const int* m, const int* n, const int* k,
                     const float* alpha, const float* d_a, const int* lda, const float* d_b, const int* ldb,
                     const float* beta, float* d_c, const int* ldc, void* stream);
int gbs_dtrsm(const char* side, const char* uplo, const char* transa, const char* diag, const int* m, const int* n,
              const double* alpha, const double* a, const int* lda, double* b, const int* ldb);
int gbs_strsm(const char* side, const char* uplo, const char* transa, const char* diag, const int* m, const int* n,
              const float* alpha, const float* a, const int* lda, float* b, const int* ldb);
int gbs_dtrsm_device(const char* side, const char* uplo, const char* transa, const char* diag, const int* m,
                     const int* n, const double* alpha, const double* d_a, const int* lda, double* d_b,
                     const int* ldb, void* stream);
int gbs_strsm_device(const char* side, const char* uplo, const char* transa, const char* diag, const int* m,
                     const int* n, const float* alpha, const float* d_a, const int* lda, float* d_b, const int* ldb,
                     void* stream);
int gbs_dsyrk(const char* uplo, const char* trans, const int* n, const int* k, const double* alpha, const double* a,
              const int* lda, const double* beta, double* c, const int* ldc);
int gbs_ssyrk(const char* uplo, const char* trans, const int* n, const int* k, const float* alpha, const float* a,
              const int* lda, const float* beta, float* c, const int* ldc);
int gbs_dsyrk_device(const char* uplo, const char* trans, const int* n, const int* k, const double* alpha,
                     const double* d_a, const int* lda, const double* beta, double* d_c, const int* ldc, void* stream);
int gbs_ssyrk_device(const char* uplo, const char* trans, const int* n, const int* k, const float* alpha,
                     const float* d_a, const int* lda, const float* beta, float* d_c, const int* ldc, void* stream);

/* ------------------------------------------------------------------ tensor cores
 * The trailing update of the low-precision tiers as a standalone GEMM,
 * C (m x n, FP32) -= A (m x k) * B (k x n), all column-major on the device,
 * on the tcgen05 tensor cores with FP32 accumulation.  Replaces, for the
 * mixed tiers, the products A22 -= A21*A12 (PartialPivLU.h:492) and
 * A22 -= A21*A21^T (LLT.h:357, lower != 0: only the lower triangle of C is
 * written, B must then be A^T and m == n).  kind: operand rounding. */
typedef enum gbs_tc_kind {
  GBS_TC_BF16 = 0,    /* bfloat16 operands */
  GBS_TC_FP16 = 1,    /* float16 operands (caller scales against overflow) */
  GBS_TC_TF32 = 2,    /* tf32 operands */
  GBS_TC_TF32X3 = 3   /* FP32 operands split hi+lo: hi*hi + hi*lo + lo*hi (FP32 accuracy) */
} gbs_tc_kind;
int gbs_tc_gemm_sub(int kind, int m, int n, int k, const float* d_a, int64_t lda, const float* d_b, int64_t ldb,
                    float* d_c, int64_t ldc, int lower, void* stream);

/* ------------------------------------------------------------------ mixed precision
 * A x = B for an FP64 matrix, factored in a low precision on the tensor cores
 * and refined in FP64 until the normwise backward error
 * max_j ||b_j - A x_j||_inf / (||A||_inf ||x_j||_inf + ||b_j||_inf) <= tol.
 * The reference has no such path; these extend PartialPivLU::solve
 * (PartialPivLU.h:224-244) and LLT::solve (LLT.h:477-505) the way LAPACK's
 * dsgesv / dsposv extend dgesv / dposv.  Refinement is classic (x += M^-1 r)
 * or GMRES-IR (each correction solves M^-1 A d = M^-1 r by GMRES in FP64 with
 * the low-precision factors applied in FP32).  When the refinement stops
 * improving, needs more than max_iter steps, or the low-precision
 * factorization breaks down, the plain FP64 factorization (the reference's
 * pivots / failing column) decides the result. */
typedef enum gbs_tier {
  GBS_TIER_FP64 = 0,     /* plain FP64 (no refinement) */
  GBS_TIER_TF32X3 = 1,   /* FP32-accurate factors: 3xTF32 tensor-core updates */
  GBS_TIER_TF32 = 2,     /* TF32 tensor-core updates */
  GBS_TIER_BF16 = 3,     /* BF16 tensor-core updates */
  GBS_TIER_FP16 = 4      /* FP16 tensor-core updates (SPD: on the unit-diagonal scaled matrix) */
} gbs_tier;

typedef enum gbs_refine_mode { GBS_REFINE_AUTO = 0, GBS_REFINE_CLASSIC = 1, GBS_REFINE_GMRES = 2 } gbs_refine_mode;
/* FP64 residuals r = b - A x of the refinement:
 *  GBS_RESID_FP64:  FP64 fused multiply-adds (the DFMA rate bounds it);
 *  GBS_RESID_OZAKI: the Ozaki scheme on the bf16 tensor cores -- A and x cut
 *     into 8 integer digit slices of 7 bits per row / column, every slice
 *     product exact in FP32 over 1024-long chunks, folded in FP64; as accurate
 *     as an FP64 GEMV (no rounding beyond 56 bits of each row's and column's
 *     maximum) at 16 n^2 bytes of device memory for the slices of A;
 *  GBS_RESID_AUTO:  Ozaki from n = 1024, FP64 below. */
typedef enum gbs_residual_mode { GBS_RESID_AUTO = 0, GBS_RESID_FP64 = 1, GBS_RESID_OZAKI = 2 } gbs_residual_mode;
/* Row pivoting of the mixed-precision LU's panels:
 *  GBS_PIVOT_TOURNAMENT: tournament pivoting (CALU, Grigori, Demmel & Xiang
 *     2011) -- every CTA of the panel's cluster proposes 32 rows by partial
 *     pivoting on its own rows, one CTA picks the panel's pivots among them;
 *     two cluster barriers per 32-column panel instead of 32, but three
 *     32-step eliminations (the CTAs', the final one, the rows of L) instead
 *     of one: on GB300 a panel's time is its per-step CTA work, not its
 *     cluster barriers, so it measures slower (84 against 57 us per panel at
 *     n = 8192), and its larger growth factor costs accuracy and, with
 *     16-bit factors, GMRES iterations.
 *  GBS_PIVOT_PARTIAL: the reference's partial pivoting (PartialPivLU's pivot
 *     order).
 *  GBS_PIVOT_AUTO: partial pivoting.
 * The refinement and its FP64 fallback guard the result whichever is used. */
typedef enum gbs_pivoting { GBS_PIVOT_AUTO = 0, GBS_PIVOT_TOURNAMENT = 1, GBS_PIVOT_PARTIAL = 2 } gbs_pivoting;

typedef struct gbs_refine_options {
  int tier;               /* gbs_tier */
  int refine;             /* gbs_refine_mode; AUTO = classic for TF32X3, GMRES-IR otherwise */
  double tol;             /* backward-error target (default 1e-13) */
  int max_iter;           /* outer refinement steps before the FP64 fallback (default 30) */
  int gmres_restart;      /* Krylov vectors per GMRES-IR correction (default 40) */
  double gmres_tol;       /* relative target of one GMRES correction (default 1e-10) */
  double shift_factor;    /* SPD tiers: diagonal shift = shift_factor * u of the tier (default 4) */
  int residual;           /* gbs_residual_mode of the FP64 residuals (default GBS_RESID_AUTO) */
  int pivoting;           /* gbs_pivoting of the general-A panels (default GBS_PIVOT_AUTO) */
  int lookahead;          /* general A: 1 (default) factors each 128-column block's panels on a second
                             stream while a third applies the previous block's wide trailing update,
                             in two disjoint SM partitions (green contexts: 64 SMs for the panels,
                             whose 16-CTA clusters then always find their GPC, the rest for the
                             update; plain streams when the driver cannot partition); 0 runs every
                             step on the caller's stream.  Same results either way. */
} gbs_refine_options;

typedef struct gbs_refine_info {
  int tier_used;          /* gbs_tier that produced X (GBS_TIER_FP64 after a fallback) */
  int solver;             /* gbs_refine_mode used */
  int iterations;         /* outer refinement steps */
  int inner_iterations;   /* GMRES iterations, summed over outer steps */
  int fell_back;          /* 1 when the FP64 factorization produced X */
  int singular;           /* 1 when the FP64 factorization met a zero pivot (LU) / non-SPD column (LLT) */
  double backward_error;  /* normwise backward error of X, computed in FP64 */
  double shift;           /* SPD tiers: diagonal shift used for the factorization */
} gbs_refine_info;

void gbs_refine_options_default(gbs_refine_options* opt);

/* R = B - A X (d_b NULL: R = A X) for an n x n FP64 matrix and nrhs columns,
 * device buffers, with the refinement's residual kernels (method: a
 * gbs_residual_mode).  Returns when R is final. */
int gbs_dgeresid_device(int n, int nrhs, const double* d_a, int lda, const double* d_x, int ldx, const double* d_b,
                        int ldb, double* d_r, int ldr, int method, void* stream);

/* General A (PartialPivLU).  Device buffers, stream-ordered on `stream`
 * (a cudaStream_t; NULL is the legacy default stream, as in every other
 * `void* stream` argument of this header); returns when X is final.  opt
 * NULL: defaults. */
int gbs_dgesv_mixed_device(int n, int nrhs, const double* d_a, int lda, const double* d_b, int ldb, double* d_x,
                           int ldx, const gbs_refine_options* opt, gbs_refine_info* info, void* stream);
/* Host buffers (copied in and out inside the call).  For 2048 <= n <= 20480,
 * nrhs <= 16 and look-ahead on, A crosses in column chunks that the
 * factorization takes in as they land (pinned host memory lets the copies
 * overlap it); the results are bit-identical to gbs_dgesv_mixed_device's on the
 * same A. */
int gbs_dgesv_mixed(int n, int nrhs, const double* a, int lda, const double* b, int ldb, double* x, int ldx,
                    const gbs_refine_options* opt, gbs_refine_info* info);
/* SPD A, lower triangle read (LLT<MatrixXd, Lower>).  Returns
 * GBS_NUMERICAL_ISSUE (info->singular = 1) when A is not positive definite in
 * FP64 either. */
int gbs_dposv_mixed_device(int n, int nrhs, const double* d_a, int lda, const double* d_b, int ldb, double* d_x,
                           int ldx, const gbs_refine_options* opt, gbs_refine_info* info, void* stream);
/* The column chunks gbs_dgesv_mixed copies A in, for order n (a diagnostic;
 * no GPU work).  Returns the number of chunks m (0: A is copied whole), fills
 * col[0..m] (chunk j holds the columns [col[j], col[j+1])) and iter[0..m-1]
 * (the look-ahead iteration at which chunk j joins the wide updates, or, for
 * the rolling chunk, at which it is gathered), and *rolling (the rolling
 * chunk's index, or -1).  col holds cap + 1 entries and iter cap; entries
 * beyond them are not written.  Any pointer may be NULL. */
int gbs_streamed_input_plan(int n, int cap, int* col, int* iter, int* rolling);
/* Host buffers: only the lower trapezoid of each 512-column block of A is
 * copied (the strict upper triangle is never read, as in LLT). */
int gbs_dposv_mixed(int n, int nrhs, const double* a, int lda, const double* b, int ldb, double* x, int ldx,
                    const gbs_refine_options* opt, gbs_refine_info* info);

/* ------------------------------------------------------------------ batched
 * Many small, uneven systems, one right-hand side each: LLT + solve for SPD
 * matrices (kind 0) and PartialPivLU + solve for general ones (kind 1), n in
 * [1, 64].  The reference has no batch API; each item gives the results of
 * LLT<MatrixX?>(A).solve(b) (LLT.h:305-328, 477-505) or
 * PartialPivLU<MatrixX?>(A).solve(b) (PartialPivLU.h:365-409, 224-244) with
 * the reference's pivot sequence and failing column.
 *
 * A plan fixes sizes and kinds; the caller's buffers hold the matrices back to
 * back (column-major, ld = n, item i at the element offset
 * sum_{j<i} n_j^2) and the right-hand sides back to back (offset
 * sum_{j<i} n_j); gbs_batched_offsets returns both offset lists.  Solving
 * overwrites the matrices with their factors (LLT: lower triangle; LU: L\U),
 * the right-hand sides with the solutions, writes info[i] (-1 = success,
 * else the failing column (LLT) or first exactly-zero pivot (LU)) and, for LU
 * items, the 0-based transpositions at the item's right-hand-side offset of
 * d_piv.  A failed LLT item (info >= 0) keeps its right-hand side; its
 * columns left of the failing one hold L, the rest is unspecified (the
 * reference's blocked LLT, n >= 32, leaves the failing block partly updated).
 * With use_graph != 0 the launch is a CUDA graph replayed per call
 * (re-captured when the buffer pointers change). */
typedef struct gbs_batched gbs_batched;
int gbs_batched_create(gbs_batched** out, int dtype, int64_t count, const int* sizes, const int* kinds,
                       int use_graph);
int gbs_batched_destroy(gbs_batched* plan);
int64_t gbs_batched_matrix_elements(const gbs_batched* plan);
int64_t gbs_batched_rhs_elements(const gbs_batched* plan);
int gbs_batched_offsets(const gbs_batched* plan, int64_t* a_offsets, int64_t* b_offsets);
int gbs_batched_solve(gbs_batched* plan, void* d_a, void* d_b, int* d_info, int* d_piv, void* stream);
/* The same solve from host buffers: a and b (read only; the factors stay on
 * the device), the solutions into x (may be b), info and piv (may be NULL),
 * in the layouts above.  A large batch is split into up to four parts of
 * consecutive items; each part crosses to the device while the previous one
 * is solved and back while the next one is (with pinned host memory).  Every
 * item is solved by the same kernel as in gbs_batched_solve, with the same
 * results.  Returns once b, info and piv are written. */
int gbs_batched_solve_host(gbs_batched* plan, const void* a, const void* b, void* x, int* info, int* piv);
/* The plan groups the items into buckets by kind and size class (LLT: n <= 8,
 * 12, 16, 20, 24, 32, 64; LU: n <= 8, 12, 16, 24, 32, 48, 64).  Each bucket
 * runs one variant: G lanes per system (G in {1, 2, 4, 8, 16}; 32 / G systems
 * per warp, one warp per CTA) or one warp per system (lanes = 32, 1-8 warps
 * per CTA); the buckets run concurrently.  gbs_batched_autotune searches the
 * variants bucket by bucket (coordinate descent), timing the whole batch on
 * the given buffers, each run from the buffers' input (kept in a scratch
 * copy; the buffers hold it again on return); a variant is kept when it
 * lowers the batch's time by more than 1 %.  With persist != 0 the choices
 * are appended to the autotune cache ($GBS_AUTOTUNE_CACHE, default
 * ~/.gb300solve_autotune.jsonl), keyed by (GPU, kind, size class, dtype);
 * later plans start from the cached choice. */
int gbs_batched_autotune(gbs_batched* plan, void* d_a, void* d_b, int* d_info, int* d_piv, int persist);
/* warps per CTA of the first bucket with n <= 32 and the first with n > 32 */
int gbs_batched_config(const gbs_batched* plan, int* warps_small, int* warps_large);
/* *count = number of buckets; desc gets min(capacity, *count) records of 7
 * ints: kind, smallest and largest n of the class, items, largest n present,
 * lanes per system, warps per CTA. */
int gbs_batched_buckets(const gbs_batched* plan, int capacity, int* count, int* desc);
/* Forces bucket i's variant (GBS_INVALID_ARGUMENT if it is not allowed for
 * the bucket or does not fit in shared memory). */
int gbs_batched_set_variant(gbs_batched* plan, int bucket, int lanes_per_system, int warps_per_cta);

/* ------------------------------------------------------------------ medium batches + precision router
 * Batches of general systems with n in [1, 512], one CTA per matrix, packed
 * back to back like gbs_batched (matrix i at sum_{j<i} n_j^2, vectors at
 * sum_{j<i} n_j).  No counterpart in the reference, which factors one matrix
 * per PartialPivLU object; each item reproduces PartialPivLU (pivots:
 * PartialPivLU.h:365-409), its solve and rcond() (ConditionEstimator.h:56-169).
 *   gbs_mbatch_lu_rcond  FP64 LU in place, 0-based pivots, solve of d_rhs in
 *                        place (may be NULL), rcond per item (d_rcond may be
 *                        NULL: not estimated), info = first zero pivot or -1
 *   gbs_mbatch_ir        FP32 LU of a working copy (d_work: matrix-sized FP32
 *                        scratch) + FP64 refinement of x to backward error
 *                        <= tol; status = refinement steps, -1 when the bound
 *                        was not reached, -2 when the FP32 factorization hit a
 *                        zero pivot (solve those items in FP64); x is written
 *                        only for the items that reached it.  factored != 0
 *                        reuses the FP32 factors already in d_work / d_piv and
 *                        refines the items whose d_status is -1
 *   gbs_mbatch_gmres_ir  the same FP32 LU as the preconditioner of FP64 GMRES
 *                        (restart <= 16, CGS2 Arnoldi) inside FP64 refinement
 *                        (GMRES-IR): at most max_outer cycles; factored and
 *                        status as for gbs_mbatch_ir (so the items a
 *                        gbs_mbatch_ir call left at -1 can be passed on as
 *                        they are); d_inner (may be NULL) = GMRES iterations
 *                        per item; the Krylov basis is held by the plan
 *                        (allocated on the first call)
 *   gbs_mbatch_features  gbs_router_feature_count() floats per item: size,
 *                        diagonal and row-norm statistics, four power-iteration
 *                        estimates of ||A||_2 / ||A||_F and their ratios
 * The router network is a 3-layer MLP (in -> 64 -> 64 -> 1, ReLU) trained on
 * the GPU by its own kernels (Adam on the mean squared error of the predicted
 * log10 condition number against rcond-derived labels); gbs_router_route maps
 * predictions to tiers: 1 = FP32 + refinement (prediction <= t_ir), 2 = FP32 +
 * GMRES-IR (<= t_gmres), 0 = FP64.
 * d_items (device, n_items indices) restricts a call to those items; NULL
 * processes every item.  Per-item outputs (info, rcond, status, features) are
 * indexed by item, so a subset call leaves the other items' entries alone. */
typedef struct gbs_mbatch gbs_mbatch;
int gbs_mbatch_create(gbs_mbatch** out, int64_t count, const int* sizes);
int gbs_mbatch_destroy(gbs_mbatch* plan);
int64_t gbs_mbatch_matrix_elements(const gbs_mbatch* plan);
int64_t gbs_mbatch_vector_elements(const gbs_mbatch* plan);
int gbs_mbatch_offsets(const gbs_mbatch* plan, int64_t* a_offsets, int64_t* v_offsets);
int gbs_mbatch_lu_rcond(gbs_mbatch* plan, const int* d_items, int64_t n_items, double* d_a, int* d_piv,
                        double* d_rhs, double* d_rcond, int* d_info, void* stream);
int gbs_mbatch_ir(gbs_mbatch* plan, const int* d_items, int64_t n_items, const double* d_a, float* d_work, int* d_piv,
                  const double* d_rhs, double* d_x, double tol, int max_iter, int factored, int* d_status,
                  void* stream);
int gbs_mbatch_gmres_ir(gbs_mbatch* plan, const int* d_items, int64_t n_items, const double* d_a, float* d_work,
                        int* d_piv, const double* d_rhs, double* d_x, double tol, int max_outer, int restart,
                        int factored, int* d_status, int* d_inner, void* stream);
int gbs_mbatch_features(gbs_mbatch* plan, const int* d_items, int64_t n_items, const double* d_a, float* d_features,
                        void* stream);
int gbs_router_feature_count(void);

typedef struct gbs_mlp gbs_mlp;
int gbs_mlp_create(gbs_mlp** out, int in_dim, int width, uint64_t seed);   /* width must be 64, in_dim <= 16 */
int gbs_mlp_destroy(gbs_mlp* mlp);
int gbs_mlp_param_count(const gbs_mlp* mlp);
int gbs_mlp_get_params(const gbs_mlp* mlp, float* host_params);
int gbs_mlp_set_params(gbs_mlp* mlp, const float* host_params);           /* also resets Adam state */
/* Gradient of mean((y - t)^2) over `count` samples (device X: count x in_dim row-major, T: count). */
int gbs_mlp_gradients(gbs_mlp* mlp, const float* d_x, const float* d_t, int count, float* host_grad, double* loss);
int gbs_mlp_train_step(gbs_mlp* mlp, const float* d_x, const float* d_t, int count, float lr, double* loss);
int gbs_mlp_fit(gbs_mlp* mlp, const float* d_x, const float* d_t, int count, int epochs, int batch, float lr,
                uint64_t seed, double* final_loss);
int gbs_mlp_predict(const gbs_mlp* mlp, const float* d_x, int count, float* d_y, void* stream);
int gbs_router_route(const float* d_pred, int count, float t_ir, float t_gmres, int* d_tier, void* stream);

/* ------------------------------------------------------------------ tracing
 * The reference has no runtime tracing (bench/BenchTimer.h times whole calls
 * from the host).  Here every kernel launch is counted, and when profiling is
 * on each phase launch is bracketed by CUDA events on its stream and tagged
 * with its algorithmic flops and bytes. */
typedef enum gbs_phase {
  GBS_PHASE_PANEL = 0, GBS_PHASE_LASWP = 1, GBS_PHASE_TRSM_LU = 2, GBS_PHASE_GEMM = 3,
  GBS_PHASE_POTRF_DIAG = 4, GBS_PHASE_TRSM_LLT = 5, GBS_PHASE_SYRK = 6, GBS_PHASE_TRI_SOLVE = 7,
  GBS_PHASE_NORM = 8, GBS_PHASE_MIXED = 9, GBS_PHASE_TC_GEMM = 10, GBS_PHASE_RESIDUAL = 11,
  GBS_PHASE_BATCHED = 12, GBS_PHASE_ROUTER = 13, GBS_PHASE_COPY = 14, GBS_PHASE_COUNT = 15
} gbs_phase;
uint64_t gbs_kernel_launch_count(void);
int gbs_profile_enable(int on);
int gbs_profile_reset(void);
/* Sums, over the phase's recorded launches, device time (ms), launch count,
 * algorithmic flops and bytes.  Waits for the recorded events. */
int gbs_profile_collect(int phase, double* ms_total, int64_t* launches, double* flops, double* bytes);
/* The recorded launches in order of issue (a timeline, e.g. to see which
 * phases of two streams overlap): phase, stream (0, 1, ... in order of first
 * use), start and end in ms from the first record's start.  Writes at most cap
 * entries (any pointer may be NULL) and returns the number of records, or
 * -(100 + gbs_status) on an error.  Waits for the recorded events. */
int gbs_profile_timeline(int* phase, int* stream, double* start_ms, double* end_ms, int cap);

#ifdef __cplusplus
}
#endif

#endif /* GB300SOLVE_H */
