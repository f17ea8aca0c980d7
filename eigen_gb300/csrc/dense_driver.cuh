// Host-side drivers of the plain factor-and-solve path (declarations shared by
// the C-ABI translation unit and the mixed-precision / batched units).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <vector>

#include "gbs_common.cuh"

namespace gbs {

int ensure_device();
int device_sm_count();

// Growable device buffer; never shrinks.  A borrowed buffer is a view of
// memory someone else owns (the allocation-free LU's fixed array): reserve()
// never allocates for it and fails with GBS_INVALID_ARGUMENT when asked for
// more than it holds, and release() never frees it.
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  bool borrowed = false;
  int reserve(size_t b);
  void release();
  template <typename U> U* as() const { return (U*)p; }
  ~DevBuf() { release(); }
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
};

// Pinned host staging buffer; never shrinks.
struct HostBuf {
  void* p = nullptr;
  size_t bytes = 0;
  int reserve(size_t b);
  void release();
  ~HostBuf() { release(); }
  HostBuf() = default;
  HostBuf(const HostBuf&) = delete;
  HostBuf& operator=(const HostBuf&) = delete;
};

// Device workspace of the persistent triangular solve: ticket counter and one
// ready flag per block row (zeroed before each launch), and a timeout flag that
// stays set across launches until solve_status reads and clears it; one per
// stream of use.
struct SolveWork {
  DevBuf flags;
  DevBuf err;
  DevBuf tmp;     // row-permutation scratch of the LDLT solve
};

// Per-call workspace for the stateless (plug-in / LAPACK) entry points: a
// stream plus buffers, taken from a process-wide pool so concurrent host
// threads never share one.
struct Workspace {
  cudaStream_t stream = nullptr;
  DevBuf a, piv, status, scratch, b, vec;
  HostBuf hvec;
  SolveWork sw;
};
struct WorkspaceLease {
  Workspace* ws = nullptr;
  int status = GBS_SUCCESS;
  WorkspaceLease();
  ~WorkspaceLease();
};

// ---- plain-path drivers (device pointers, stream-ordered; the status word
// must be zero-initialised with info = -1 before a factorization)
int reset_status(DeviceStatus* d_st, cudaStream_t s);
// Sets the process-wide wait limit (0: the 2 s default).
void set_wait_limit_ns(uint64_t ns);
// Failure-detection diagnostics: one launch each whose wait never succeeds;
// both return GBS_TIMEOUT when the wait expired and the launch ended.
int tri_solve_timeout_selftest(cudaStream_t s, int n);
int barrier_timeout_selftest(cudaStream_t s);
int read_status(const DeviceStatus* d_st, DeviceStatus* h_st, cudaStream_t s);

constexpr int kPanelNB = 32;   // columns factored per panel launch

// Unblocked partial-pivoting LU of the m x nbc panel at `a` (nbc <= kPanelNB);
// writes absolute pivot rows k0 + p into tr[0..nbc).  With map_out, may also
// leave the interchanges as a device row map for laswp_map_apply (*map_out
// is null when it did not).  With trsm_done, may also interchange the
// trsm_cols columns right of the panel and solve their top rows with L11
// (*trsm_done says whether it did; the caller then skips those columns).
// tournament: the mixed-precision path's panels may take tournament pivoting
// (panel_lu_tournament_kernel) instead of the reference's partial pivoting.
template <typename T>
int panel_factor(cudaStream_t s, T* a, int64_t lda, int m, int nbc, int k0, int* tr, DevBuf& scratch,
                 DeviceStatus* st, const int** map_out = nullptr, int trsm_cols = 0, bool* trsm_done = nullptr,
                 bool tournament = false);
// CTAs of the cluster panel_factor launches for a panel of m rows (one per SM).
int panel_cluster_ctas(int m);

constexpr int kLaswpMapInts = 520;     // count, 256 target rows, 256 source rows (+ pad)

// Applies a row map (as written by laswp_map_kernel or the cluster panel) to
// the columns [c0, c1) and [c2, c3) of A, all SMs.
template <typename T>
int laswp_map_apply(cudaStream_t s, T* A, int64_t lda, const int* map, int c0, int c1, int c2, int c3);

template <typename T>
int getrf_device(cudaStream_t s, int m, int n, T* dA, int64_t lda, int* dTr, DeviceStatus* dSt, DevBuf& scratch);

// Loads every kernel getrf_device<T> can launch, for any shape, and runs its
// one-time capacity queries.  CUDA loads kernels lazily on their first launch,
// and loading one can take device memory; a caller that must not allocate
// later runs this once per device beforehand.  panel_preload<T> does the same
// for the panel kernels (their own translation unit).
template <typename T>
int getrf_preload();
template <typename T>
int panel_preload();

template <typename T>
int potrf_device(cudaStream_t s, int n, T* dA, int64_t lda, int upper, DeviceStatus* dSt, DevBuf& tmp);

// op(Tri) X = B in place on B (n x nrhs, ldb).  lower: which triangle of tri
// holds the factor; trans: solve with its transpose; unit: unit diagonal.
template <typename T>
int tri_solve_device(cudaStream_t s, int n, int nrhs, const T* tri, int64_t ld, int lower, int trans, int unit,
                     T* B, int64_t ldb, SolveWork& w, const T* dinv = nullptr);

// Block height of tri_solve_device's persistent kernel (its dinv blocks are
// NB x NB).  A block step costs a fixed flag-to-flag latency plus work that
// grows with NB^2: FP32 64-row blocks beat both 32 and 128 at n = 8192.
template <typename T>
constexpr int tri_solve_nb() { return sizeof(T) == 8 ? 32 : 64; }

// Waits for the stream and reports GBS_TIMEOUT if a solve's wait expired.
int solve_status(cudaStream_t s, SolveWork& w);
// Allocates (zeroed) the timeout flag solve_status reads, if not yet there.
int solve_err_slot(cudaStream_t s, SolveWork& w);

template <typename T>
int laswp_device(cudaStream_t s, T* B, int64_t ldb, int ncols, const int* dTr, int i0, int i1, int reverse);

// A x = b with PA = LU (transpose: A^T x = b), in place on B.
template <typename T>
int lu_solve_device(cudaStream_t s, int n, int nrhs, const T* dLU, int64_t ld, const int* dTr, T* B, int64_t ldb,
                    int transpose, SolveWork& w);

template <typename T>
int llt_solve_device(cudaStream_t s, int n, int nrhs, const T* dL, int64_t ld, int upper, T* B, int64_t ldb,
                     SolveWork& w);

template <typename T>
int l1_norm_device(cudaStream_t s, const T* dA, int64_t lda, int m, int n, int sym, int upper, double* d_out,
                   double* h_out);

// Hager/Higham estimate of ||A^{-1}||_1 (ConditionEstimator.h:56-142); kind 3 =
// LDLT (dF the lower factor of the permuted matrix, dTr its row order), kind 0 = LU,
// 1 = LLT lower, 2 = LLT upper.  `vec` holds 2n scalars of device scratch.
template <typename T>
int inv_l1_estimate_device(cudaStream_t s, int kind, int n, const T* dF, int64_t ld, const int* dTr,
                           DevBuf& vec, HostBuf& hvec, SolveWork& w, double* est);

double rcond_from_estimate(int64_t n, double matrix_norm, double inv_norm, bool single);

template <typename T>
int copy_matrix_device(cudaStream_t s, const T* a, int64_t lda, T* b, int64_t ldb, int m, int n);

// C -= op(A) op(B) on the SIMT cores (strided operands, see gemm_sub_kernel).
template <typename T>
int gemm_sub_device(cudaStream_t s, int phase, int M, int N, int K, const T* A, int64_t a_rs, int64_t a_cs, const T* B,
                    int64_t b_rs, int64_t b_cs, T* C, int64_t ldc);

// Lower triangle of C (n x n) -= op(A) op(B) (the SYRK form of gemm_sub_device).
template <typename T>
int syrk_sub_device(cudaStream_t s, int phase, int n, int K, const T* A, int64_t a_rs, int64_t a_cs, const T* B,
                    int64_t b_rs, int64_t b_cs, T* C, int64_t ldc);

// LDLT solve (LDLT.h:540-577) on the lower factor W (unit L strictly below the
// diagonal, D on it, ld) of the symmetrically permuted matrix; perm[i] = the
// original row at position i.  In place on B (n x nrhs).
template <typename T>
int ldlt_solve_device(cudaStream_t s, int n, int nrhs, const T* W, int64_t ld, const int* perm, T* B, int64_t ldb,
                      SolveWork& w);

// LLT::rankUpdate (LLT.h:231-299) on the factor in A (lower, or the upper
// triangle read as the transposed view), v on the device; *failed = the first
// column whose downdated diagonal would not be positive, or -1.  Waits for it.
template <typename T>
int llt_rank_update_device(cudaStream_t s, int n, T* A, int64_t lda, int upper, const T* d_v, double sigma,
                           DevBuf& tmp, int* failed);

// B(kb x ncols) <- L^{-1} B, L unit lower with kb <= 128 rows and many columns.
template <typename T>
int trsm_lunit_wide(cudaStream_t s, int kb, int ncols, const T* L, int64_t ldl, T* B, int64_t ldb);

// Row interchanges tr[i0..i1) (in order, at most 128) on columns [c0,c1) and
// [c2,c3) as one gather per column; `map` is a small device scratch.
template <typename T>
int laswp_gather_device(cudaStream_t s, T* A, int64_t lda, const int* tr, int i0, int i1, int c0, int c1, int c2,
                        int c3, DevBuf& map);
// The same for the interchanges of one outer block (at most 128, rows in
// [i0, m)): the row map is built in shared memory in constant time per
// interchange (falls back to laswp_gather_device when [i0, m) is too tall).
constexpr size_t kBlockMapSmemMax = 160 * 1024;
template <typename T>
int laswp_block_device(cudaStream_t s, T* A, int64_t lda, int m, const int* tr, int i0, int i1, int c0, int c1,
                       int c2, int c3, DevBuf& map);

}  // namespace gbs
