// Mixed-precision factorizations + FP64 refinement (the LAPACK dsgesv /
// dsposv idea, with the trailing updates on the tcgen05 tensor cores).
//
// Factorizations (FP32 working storage, tensor-core updates in the tier's
// precision: BF16 / FP16 / TF32 / 3xTF32):
//   mixed_getrf  P A = L U: 128-column outer panels, each factored 32 columns
//                at a time by the panel kernel; the outer U12 = L11^-1 A12 as
//                A12 - (I - L11^-1) A12 on tensor cores (explicit inverse of
//                the unit-lower diagonal block); inner and outer trailing
//                updates A22 -= A21 A12 on tensor cores; with look-ahead the
//                panels of block k+1 run on a second stream during block k's
//                wide trailing update
//   mixed_potrf  D A D + sigma I = L L^T, D = diag(A)^-1/2 (unit diagonal, so
//                FP16 cannot overflow), the reference's block size; diagonal
//                blocks and TRSM on FP32 cores, SYRK on tensor cores
// Refinement (FP64 residuals against the original matrix):
//   classic IR   x += M^-1 r until the normwise backward error
//                max_j ||r_j||_inf / (||A||_inf ||x_j||_inf + ||b_j||_inf) <= tol
//   GMRES-IR     each correction solves M^-1 A d = M^-1 r with GMRES
//                (CGS2 orthogonalisation, FP64), preconditioner applied in
//                FP32 (Carson & Higham, SIAM J. Sci. Comput. 40(2), 2018)
// A refinement whose backward error stops halving, or a low-precision
// factorization that breaks down, falls back to the plain FP64 factorization.
#include <algorithm>
#include <cmath>
#include <mutex>
#include <vector>

#include "dense_driver.cuh"
#include "dense_kernels.cuh"
#include "gbs_profile.cuh"
#include "mixed_driver.cuh"
#include "ozaki.cuh"
#include "tc_gemm.cuh"

namespace gbs {

static inline int cdiv(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }

// ------------------------------------------------------------------ kernels
// Y = A X (B == null) or R = B - A X, FP64.  Grid (row blocks of 128, K
// splits); a thread owns one row and RC right-hand sides (RC = 4, 8 or 16,
// the smallest that covers nrhs, so no FMA is spent on absent columns); the
// K-chunk of X is staged in shared memory.  A is read column by column,
// coalesced over rows.  Partial sums per split are added in split order by
// residual_reduce (deterministic).
constexpr int kResRows = 128, kResRC = 16, kResKC = 64;
constexpr int kMixedNB = 128;                  // outer block width of the mixed LU
constexpr int kInflowMaxChunks = 16;           // column chunks of the streamed host input (LU)
constexpr int kOzakiMinN = 1024;      // GBS_RESID_AUTO: tensor-core residuals from this order

template <int RC>
__global__ void __launch_bounds__(kResRows)
mv_partial_kernel(int n, int nrhs, const double* __restrict__ A, int64_t lda, const double* __restrict__ X,
                  int64_t ldx, int kspan, double* __restrict__ part)
{
  __shared__ double sx[kResKC][RC];
  const int row = blockIdx.x * kResRows + threadIdx.x;
  const int split = blockIdx.y;
  const int k0 = split * kspan, k1 = min(n, k0 + kspan);
  double acc[RC];
#pragma unroll
  for (int c = 0; c < RC; ++c) acc[c] = 0.0;
  for (int kc = k0; kc < k1; kc += kResKC) {
    __syncthreads();
    for (int e = threadIdx.x; e < kResKC * RC; e += kResRows) {
      const int kk = e % kResKC, c = e / kResKC;
      sx[kk][c] = (kc + kk < k1 && c < nrhs) ? X[(int64_t)c * ldx + kc + kk] : 0.0;
    }
    __syncthreads();
    if (row < n) {
      const int kend = min(kResKC, k1 - kc);
      const double* ap = A + (int64_t)kc * lda + row;
#pragma unroll 4
      for (int kk = 0; kk < kend; ++kk) {
        const double a = ap[(int64_t)kk * lda];
#pragma unroll
        for (int c = 0; c < RC; ++c) acc[c] = fma(a, sx[kk][c], acc[c]);
      }
    }
  }
  if (row < n) {
    for (int c = 0; c < nrhs && c < RC; ++c) part[((int64_t)split * nrhs + c) * n + row] = acc[c];
  }
}

// Full symmetric copy of the lower triangle: F(i,j) = A(max,min), by 32x32
// tiles through shared memory so both the read and the write are coalesced.
__global__ void symmetrize_kernel(int n, const double* __restrict__ A, int64_t lda, double* __restrict__ F)
{
  __shared__ double t[32][33];
  const int bi = blockIdx.x * 32, bj = blockIdx.y * 32;
  if (bi < bj) {
    // upper tile (bi, bj): transpose of the lower tile (bj, bi)
    for (int y = threadIdx.y; y < 32; y += 8) {
      const int r = bj + threadIdx.x, c = bi + y;
      t[y][threadIdx.x] = (r < n && c < n) ? A[(int64_t)c * lda + r] : 0.0;
    }
    __syncthreads();
    for (int y = threadIdx.y; y < 32; y += 8) {
      const int r = bi + threadIdx.x, c = bj + y;
      if (r < n && c < n) F[(int64_t)c * n + r] = t[threadIdx.x][y];
    }
  } else {
    for (int y = threadIdx.y; y < 32; y += 8) {
      const int r = bi + threadIdx.x, c = bj + y;
      if (r < n && c < n) F[(int64_t)c * n + r] = r >= c ? A[(int64_t)c * lda + r] : A[(int64_t)r * lda + c];
    }
  }
}

__global__ void residual_reduce_kernel(int n, int nrhs, int splits, const double* __restrict__ part,
                                       const double* __restrict__ B, int64_t ldb, double* __restrict__ R, int64_t ldr)
{
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)n * nrhs) return;
  const int row = (int)(t % n), c = (int)(t / n);
  double s = 0.0;
  for (int k = 0; k < splits; ++k) s += part[((int64_t)k * nrhs + c) * n + row];
  R[(int64_t)c * ldr + row] = B ? B[(int64_t)c * ldb + row] - s : s;
}

// out[which*nrhs + c] = max_i |V(i, c)| for V = R, X, B (which = 0, 1, 2)
__global__ void col_absmax3_kernel(int n, int nrhs, const double* R, int64_t ldr, const double* X, int64_t ldx,
                                   const double* B, int64_t ldb, double* out)
{
  const int which = blockIdx.y;
  const int c = blockIdx.x;
  const double* V = which == 0 ? R : which == 1 ? X : B;
  const int64_t ld = which == 0 ? ldr : which == 1 ? ldx : ldb;
  double m = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    double v = fabs(V[(int64_t)c * ld + i]);
    m = (v > m || v != v) ? v : m;
  }
  m = warp_max(m);
  __shared__ double sm[32];
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    m = threadIdx.x < (blockDim.x >> 5) ? sm[threadIdx.x] : 0.0;
    m = warp_max(m);
    if (threadIdx.x == 0) out[which * nrhs + c] = m;
  }
}

// ||A||_inf rows: general (sym = 0) or symmetric with the lower triangle stored
__global__ void row_abs_sum_kernel(int n, const double* __restrict__ A, int64_t lda, int sym, double* __restrict__ rows)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0.0;
  if (!sym) {
    for (int j = 0; j < n; ++j) s += fabs(A[(int64_t)j * lda + i]);
  } else {
    for (int j = 0; j <= i; ++j) s += fabs(A[(int64_t)j * lda + i]);
    for (int j = i + 1; j < n; ++j) s += fabs(A[(int64_t)i * lda + j]);
  }
  rows[i] = s;
}

// Row sums of |A| (general A) over the column range [k0, k0 + kspan) of
// blockIdx.y, one thread per row: part[blockIdx.y][i].  Summed over the ranges
// in a fixed order by row_abs_reduce_kernel, so the norm is deterministic.
__global__ void row_abs_partial_kernel(int n, const double* __restrict__ A, int64_t lda, int kspan,
                                       double* __restrict__ part)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int k0 = blockIdx.y * kspan, k1 = min(n, k0 + kspan);
  double s0 = 0.0, s1 = 0.0;
  int k = k0;
  for (; k + 1 < k1; k += 2) {                       // two independent chains
    s0 += fabs(A[(int64_t)k * lda + i]);
    s1 += fabs(A[(int64_t)(k + 1) * lda + i]);
  }
  if (k < k1) s0 += fabs(A[(int64_t)k * lda + i]);
  part[(int64_t)blockIdx.y * n + i] = s0 + s1;
}

__global__ void row_abs_reduce_kernel(int n, int splits, const double* __restrict__ part, double* __restrict__ rows)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0.0;
  for (int k = 0; k < splits; ++k) s += part[(int64_t)k * n + i];
  rows[i] = s;
}

// W32 = fp32(R / s_c), s_c = max_i |R(i,c)| (1 when zero); W packed n x nrhs
// W = R / s_c in FP32; with perm, rows are gathered: W(i) = R(perm[i]) / s_c
// (the row interchanges of P A = L U applied on the way)
__global__ void scale_to_f32_kernel(int n, int nrhs, const double* __restrict__ R, int64_t ldr,
                                    const double* __restrict__ scale, float* __restrict__ W,
                                    const int* __restrict__ perm)
{
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)n * nrhs) return;
  const int row = (int)(t % n), c = (int)(t / n);
  const double s = scale[c] > 0.0 ? scale[c] : 1.0;
  W[t] = (float)(R[(int64_t)c * ldr + (perm ? perm[row] : row)] / s);
}

// perm = the row order of P from the transpositions tr[0..n) (applied in
// order to the identity, PermutationMatrix.h:82-88): x = P b is x(i) = b(perm[i]).
// One CTA; the index array lives in shared memory, one warp applies the swaps.
__global__ void perm_from_transpositions_kernel(int n, const int* __restrict__ tr, int* __restrict__ perm)
{
  extern __shared__ int sp[];
  for (int i = threadIdx.x; i < n; i += blockDim.x) sp[i] = i;
  __syncthreads();
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    for (int k0 = 0; k0 < n; k0 += 32) {
      const int pl = k0 + lane < n ? tr[k0 + lane] : 0;
      const int cnt = min(32, n - k0);
      for (int q = 0; q < cnt; ++q) {
        const int p = __shfl_sync(0xffffffffu, pl, q);
        if (lane == 0 && p != k0 + q) {
          const int t = sp[k0 + q];
          sp[k0 + q] = sp[p];
          sp[p] = t;
        }
      }
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) perm[i] = sp[i];
}

// X = init ? s_c W : X + s_c W   (FP64)
__global__ void update_from_f32_kernel(int n, int nrhs, const float* __restrict__ W, const double* __restrict__ scale,
                                       double* __restrict__ X, int64_t ldx, int init)
{
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)n * nrhs) return;
  const int row = (int)(t % n), c = (int)(t / n);
  const double s = scale[c] > 0.0 ? scale[c] : 1.0;
  const double d = s * (double)W[t];
  double* xp = X + (int64_t)c * ldx + row;
  *xp = init ? d : *xp + d;
}

// W32 (packed n x nrhs) *= d (FP32 diagonal scaling of the LLT tier)
__global__ void diag_scale_f32_kernel(int n, int nrhs, const float* __restrict__ d, float* __restrict__ W)
{
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)n * nrhs) return;
  W[t] *= d[t % n];
}

// As32(i,j) = fp32(d_i a_ij d_j) (+ sigma on the diagonal), lower triangle;
// d_i = 1 / sqrt(a_ii).  Also writes d in FP32.
__global__ void spd_diag_kernel(int n, const double* __restrict__ A, int64_t lda, double* __restrict__ d64,
                                float* __restrict__ d32)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double d = 1.0 / sqrt(A[(int64_t)i * lda + i]);
  d64[i] = d;
  d32[i] = (float)d;
}

__global__ void scale_spd_kernel(int n, const double* __restrict__ A, int64_t lda, double sigma,
                                 const double* __restrict__ d64, float* __restrict__ As)
{
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)n * n) return;
  const int i = (int)(t % n), j = (int)(t / n);
  if (i < j) return;
  double v = d64[i] * A[(int64_t)j * lda + i] * d64[j];
  if (i == j) v += sigma;
  As[(int64_t)j * n + i] = (float)v;
}

// ---- GMRES helpers; the Krylov basis is stored as slabs V_i (n x nrhs, ld n)
// out[i*nrhs + c] = <V_i(:,c), W(:,c)>, i < k
__global__ void gmres_dots_kernel(int n, int nrhs, const double* __restrict__ V, const double* __restrict__ W,
                                  double* __restrict__ out)
{
  const int i = blockIdx.x, c = blockIdx.y;
  const double* v = V + (int64_t)i * n * nrhs + (int64_t)c * n;
  const double* w = W + (int64_t)c * n;
  double s = 0.0;
  for (int t = threadIdx.x; t < n; t += blockDim.x) s = fma(v[t], w[t], s);
  s = warp_sum(s);
  __shared__ double sm[32];
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < (blockDim.x >> 5) ? sm[threadIdx.x] : 0.0;
    s = warp_sum(s);
    if (threadIdx.x == 0) out[i * nrhs + c] = s;
  }
}

// W(:,c) += sign * sum_{i<k} coef[i*nrhs + c] V_i(:,c)   (W with leading dimension ldw)
__global__ void gmres_combine_kernel(int n, int nrhs, int k, const double* __restrict__ V,
                                     const double* __restrict__ coef, double sign, double* __restrict__ W, int64_t ldw)
{
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)n * nrhs) return;
  const int row = (int)(t % n), c = (int)(t / n);
  double s = 0.0;
  for (int i = 0; i < k; ++i) s = fma(coef[i * nrhs + c], V[(int64_t)i * n * nrhs + (int64_t)c * n + row], s);
  W[(int64_t)c * ldw + row] += sign * s;
}

// V_out(:,c) = W(:,c) * inv[c]
__global__ void gmres_scale_kernel(int n, int nrhs, const double* __restrict__ W, const double* __restrict__ inv,
                                   double* __restrict__ Vout)
{
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)n * nrhs) return;
  Vout[t] = W[t] * inv[t / n];
}

// ------------------------------------------------------------------ SM partition
// Two disjoint SM partitions of the device as green contexts (CUDA driver API,
// resolved at run time like the tensor-map encoder): 32 SMs for the look-ahead
// LU's panels, whose 16-CTA clusters must find their SMs free within one GPC,
// and the rest for the wide trailing updates.  Created once per process; when
// the driver cannot make them, the look-ahead runs on plain streams.
constexpr unsigned int kPanelPartitionSms = 64;   // the panels' cluster plus room for their block updates

struct SmPartition {
  bool ok = false;
  CUgreenCtx panel = nullptr, update = nullptr;
  int panel_sms = 0, update_sms = 0;
};

namespace {

template <typename F>
F driver_fn(const char* name)
{
  void* p = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion(name, &p, 12050, cudaEnableDefault, &q) != cudaSuccess ||   // green streams: 12.5
      q != cudaDriverEntryPointSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return (F)p;
}

typedef CUresult (*DeviceGetFn)(CUdevice*, int);
typedef CUresult (*GetDevResourceFn)(CUdevice, CUdevResource*, CUdevResourceType);
typedef CUresult (*SplitByCountFn)(CUdevResource*, unsigned int*, const CUdevResource*, CUdevResource*, unsigned int,
                                   unsigned int);
typedef CUresult (*GenerateDescFn)(CUdevResourceDesc*, CUdevResource*, unsigned int);
typedef CUresult (*GreenCtxCreateFn)(CUgreenCtx*, CUdevResourceDesc, CUdevice, unsigned int);
typedef CUresult (*GreenStreamCreateFn)(CUstream*, CUgreenCtx, unsigned int, int);

const SmPartition& sm_partition()
{
  static SmPartition part;
  static std::once_flag once;
  std::call_once(once, [] {
    auto dev_get = driver_fn<DeviceGetFn>("cuDeviceGet");
    auto get_res = driver_fn<GetDevResourceFn>("cuDeviceGetDevResource");
    auto split = driver_fn<SplitByCountFn>("cuDevSmResourceSplitByCount");
    auto gen = driver_fn<GenerateDescFn>("cuDevResourceGenerateDesc");
    auto create = driver_fn<GreenCtxCreateFn>("cuGreenCtxCreate");
    if (!dev_get || !get_res || !split || !gen || !create) return;
    int d = 0;
    if (cudaGetDevice(&d) != cudaSuccess) return;
    CUdevice dev;
    CUdevResource all, group[1], rest;
    unsigned int ngroups = 1;
    CUdevResourceDesc da, db;
    if (dev_get(&dev, d) != CUDA_SUCCESS || get_res(dev, &all, CU_DEV_RESOURCE_TYPE_SM) != CUDA_SUCCESS) return;
    if (split(group, &ngroups, &all, &rest, CU_DEV_SM_RESOURCE_SPLIT_MAX_POTENTIAL_CLUSTER_SIZE, kPanelPartitionSms) !=
            CUDA_SUCCESS ||
        ngroups != 1 || rest.sm.smCount < 64)
      return;
    if (gen(&da, group, 1) != CUDA_SUCCESS || gen(&db, &rest, 1) != CUDA_SUCCESS) return;
    if (create(&part.panel, da, dev, CU_GREEN_CTX_DEFAULT_STREAM) != CUDA_SUCCESS ||
        create(&part.update, db, dev, CU_GREEN_CTX_DEFAULT_STREAM) != CUDA_SUCCESS)
      return;
    part.panel_sms = (int)group[0].sm.smCount;
    part.update_sms = (int)rest.sm.smCount;
    part.ok = true;
  });
  return part;
}

int partition_stream(CUgreenCtx g, int priority, cudaStream_t* out)
{
  auto create = driver_fn<GreenStreamCreateFn>("cuGreenCtxStreamCreate");
  CUstream st = nullptr;
  if (!create || create(&st, g, CU_STREAM_NON_BLOCKING, priority) != CUDA_SUCCESS) {
    gbs_set_last_message("cuGreenCtxStreamCreate failed");
    return GBS_CUDA_ERROR;
  }
  *out = (cudaStream_t)st;
  return GBS_SUCCESS;
}

}  // namespace

// ------------------------------------------------------------------ workspace pool
// Streams of the look-ahead LU: the panels of block k+1 run on `side` while
// `wide` applies block k's interchanges to the other columns and its wide
// trailing update; the caller's stream does the short serial part in between.
// With an SM partition, side and wide live in its two green contexts (disjoint
// SMs); otherwise side is a highest-priority stream and wide is the caller's.
struct Lookahead {
  cudaStream_t side = nullptr, wide = nullptr;
  int wide_sms = 0;
  cudaEvent_t ready = nullptr, panels = nullptr, wide_done = nullptr, swapped = nullptr;
  TcWorkspace tc_side, tc_wide;
  DevBuf map_side, map[2], minv[2];
  DevBuf minv_all, srcmap;   // streamed input: every block's I - L11^-1; the composed row map of a join
  int init()
  {
    if (!side) {
      int least = 0, greatest = 0;
      GBS_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&least, &greatest));
      const SmPartition& part = sm_partition();
      if (part.ok && partition_stream(part.panel, greatest, &side) == GBS_SUCCESS &&
          partition_stream(part.update, 0, &wide) == GBS_SUCCESS) {
        wide_sms = part.update_sms;
      } else {
        if (side) cudaStreamDestroy(side);
        side = wide = nullptr;
        wide_sms = 0;
        GBS_CUDA_TRY(cudaStreamCreateWithPriority(&side, cudaStreamNonBlocking, greatest));
      }
    }
    if (!ready) GBS_CUDA_TRY(cudaEventCreateWithFlags(&ready, cudaEventDisableTiming));
    if (!panels) GBS_CUDA_TRY(cudaEventCreateWithFlags(&panels, cudaEventDisableTiming));
    if (!wide_done) GBS_CUDA_TRY(cudaEventCreateWithFlags(&wide_done, cudaEventDisableTiming));
    if (!swapped) GBS_CUDA_TRY(cudaEventCreateWithFlags(&swapped, cudaEventDisableTiming));
    for (int i = 0; i < 2; ++i) GBS_TRY(minv[i].reserve(sizeof(float) * kMixedNB * kMixedNB));
    return GBS_SUCCESS;
  }
  ~Lookahead()
  {
    if (ready) cudaEventDestroy(ready);
    if (panels) cudaEventDestroy(panels);
    if (wide_done) cudaEventDestroy(wide_done);
    if (swapped) cudaEventDestroy(swapped);
    if (side) cudaStreamDestroy(side);
    if (wide) cudaStreamDestroy(wide);
  }
};

// Low-priority stream for work that only the refinement needs (the digit
// slices of A), so that it runs beside the factorization.
struct AuxStream {
  cudaStream_t s = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr, norm = nullptr;
  bool pending = false;      // join recorded and not yet waited for
  int init()
  {
    if (!s) {
      int least = 0, greatest = 0;
      GBS_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&least, &greatest));
      GBS_CUDA_TRY(cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, least));
    }
    if (!fork) GBS_CUDA_TRY(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
    if (!join) GBS_CUDA_TRY(cudaEventCreateWithFlags(&join, cudaEventDisableTiming));
    if (!norm) GBS_CUDA_TRY(cudaEventCreateWithFlags(&norm, cudaEventDisableTiming));
    return GBS_SUCCESS;
  }
  // the auxiliary stream starts after `ready`, or after what s has issued so far
  int fork_from(cudaStream_t from, cudaEvent_t ready)
  {
    GBS_TRY(init());
    if (!ready) {
      GBS_CUDA_TRY(cudaEventRecord(fork, from));
      ready = fork;
    }
    GBS_CUDA_TRY(cudaStreamWaitEvent(s, ready, 0));
    return GBS_SUCCESS;
  }
  ~AuxStream()
  {
    if (norm) cudaEventDestroy(norm);
    if (fork) cudaEventDestroy(fork);
    if (join) cudaEventDestroy(join);
    if (s) cudaStreamDestroy(s);
  }
};

// The copy stream of the streamed host input and one event per chunk.
struct CopyLane {
  cudaStream_t s = nullptr;
  cudaEvent_t ev[kInflowMaxChunks] = {};
  int init()
  {
    if (!s) GBS_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    for (cudaEvent_t& e : ev)
      if (!e) GBS_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    return GBS_SUCCESS;
  }
  ~CopyLane()
  {
    for (cudaEvent_t e : ev)
      if (e) cudaEventDestroy(e);
    if (s) cudaStreamDestroy(s);
  }
};

struct MixedWork {
  cudaStream_t stream = nullptr;
  DevBuf a32, tr, st, scratch, r, part, w32, stats, rows, a64, map, d32, d64, afull, z, v, w, coef, perm, minv,
      dinv, npart;   // npart: the norm's partial sums (its stream may run beside the residuals')
  SolveWork sw;
  TcWorkspace tc;
  Lookahead la;
  OzakiMatrix oz;          // A's digit slices when the residuals run on the tensor cores
  OzakiWork ozw;
  AuxStream aux;
  CopyLane copy;
  HostBuf hstats, hrows;
};

static std::mutex g_mpool_mu;
static std::vector<MixedWork*> g_mpool;

struct MixedLease {
  MixedWork* w = nullptr;
  int status = GBS_SUCCESS;
  MixedLease()
  {
    status = ensure_device();
    if (status != GBS_SUCCESS) return;
    {
      std::lock_guard<std::mutex> lk(g_mpool_mu);
      if (!g_mpool.empty()) {
        w = g_mpool.back();
        g_mpool.pop_back();
      }
    }
    if (!w) w = new MixedWork();
  }
  ~MixedLease()
  {
    if (!w) return;
    std::lock_guard<std::mutex> lk(g_mpool_mu);
    g_mpool.push_back(w);
  }
};

static int tc_kind(int tier)
{
  return tier == GBS_TIER_BF16 ? TC_BF16 : tier == GBS_TIER_FP16 ? TC_FP16 : tier == GBS_TIER_TF32 ? TC_TF32 : TC_TF32X3;
}

// ------------------------------------------------------------------ factorizations
constexpr int kPermSmemMax = 56 * 1024;          // perm_from_transpositions_kernel: n ints of shared memory

// M = I - L^-1 for the lower nb x nb block L (nb <= kMixedNB, ld; unit != 0:
// unit diagonal, not read), M column-major with ld kMixedNB.  Recursive
// doubling over 32 x 32 diagonal blocks of X = L^-1:
//   1. each diagonal block inverted by one warp, lane j holding column j in
//      registers (substitution on the identity, no barriers);
//   2. the 64 x 64 halves: X(b, a) = -X(b, b) (L(b, a) X(a, a)) for the block
//      pairs (0, 1) and (2, 3);
//   3. the whole block: the same with the 64 x 64 halves.
// The products run on register tiles from shared memory.  One CTA of
// 4 kMixedNB threads; rows and columns beyond nb are the identity.
constexpr int kInvLd = kMixedNB + 1;
constexpr size_t kInvSmem = sizeof(float) * (2 * kMixedNB * kInvLd + 32 * kInvLd + 4 * kMixedNB);
static_assert(kMixedNB == 128, "the inverse is written for 128 x 128 blocks");

// C(r0 + i, c) = sign * sum_{k < K} A(r0 + i, k) B(k, c) for i < ROWS: A, B, C
// row-major sub-blocks in shared memory (leading dimensions lda, ldb, ldc); the
// lanes of a warp take consecutive columns c, so B and C accesses are
// conflict-free and A's are broadcasts.
template <int ROWS, int K>
__device__ __forceinline__ void smem_tile_product(const float* A, int lda, const float* B, int ldb, float* C, int ldc,
                                                  int r0, int c, float sign)
{
  float acc[ROWS];
#pragma unroll
  for (int i = 0; i < ROWS; ++i) acc[i] = 0.f;
#pragma unroll 8
  for (int k = 0; k < K; ++k) {
    const float bv = B[k * ldb + c];
#pragma unroll
    for (int i = 0; i < ROWS; ++i) acc[i] = fmaf(A[(r0 + i) * lda + k], bv, acc[i]);
  }
#pragma unroll
  for (int i = 0; i < ROWS; ++i) C[(r0 + i) * ldc + c] = sign * acc[i];
}

// X = L^-1 of the lower nb x nb block (upper != 0: of U^T for the upper block
// U at L, i.e. X = U^-T) in shared memory; see unit_lower_inverse_kernel.
__device__ void tri_inverse_smem(const float* __restrict__ L, int64_t ld, int nb, int unit, int upper, float* sm)
{
  constexpr int LD = kInvLd;
  float* Ls = sm;                                   // [128][LD]
  float* X = sm + kMixedNB * LD;                    // [128][LD]
  float* T = sm + 2 * kMixedNB * LD;                // product scratch, up to [64][65]
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int e = tid; e < kMixedNB * kMixedNB; e += blockDim.x) {
    const int r = e % kMixedNB, c = e / kMixedNB;
    const bool in = r < nb && c < nb && r >= c && (r != c || !unit);
    Ls[r * LD + c] = in ? (upper ? L[(int64_t)r * ld + c] : L[(int64_t)c * ld + r]) : (r == c ? 1.f : 0.f);
  }
  __syncthreads();
  // 1. diagonal blocks: x[i] = X(o + i, o + lane); x[k] = 0 for k < lane, so
  //    the sums may run over every k < i
  if (warp < 4) {
    const int o = 32 * warp;
    float x[32];
#pragma unroll
    for (int i = 0; i < 32; ++i) {
      float acc = (i == lane) ? 1.f : 0.f;
#pragma unroll
      for (int k = 0; k < i; ++k) acc = fmaf(-Ls[(o + i) * LD + o + k], x[k], acc);
      x[i] = acc / Ls[(o + i) * LD + o + i];
    }
#pragma unroll
    for (int i = 0; i < 32; ++i) X[(o + i) * LD + o + lane] = x[i];
    for (int i = 0; i < 32; ++i)                     // the blocks right of the diagonal are zero
      for (int cb = o + 32; cb < kMixedNB; cb += 32) X[(o + i) * LD + cb + lane] = 0.f;
  }
  __syncthreads();
  // 2. block pairs p = 0, 1 (a = 64 p, b = a + 32): T = L(b, a) X(a, a), then
  //    X(b, a) = -X(b, b) T; thread: column lane, rows 4 g .. 4 g + 3
  const int p = tid >> 8, g = (tid >> 5) & 7;
  {
    const int oa = 64 * p, ob = oa + 32;
    float* Tp = T + p * 32 * 33;
    smem_tile_product<4, 32>(Ls + ob * LD + oa, LD, X + oa * LD + oa, LD, Tp, 33, 4 * g, lane, 1.f);
    __syncthreads();
    smem_tile_product<4, 32>(X + ob * LD + ob, LD, Tp, 33, X + ob * LD + oa, LD, 4 * g, lane, -1.f);
  }
  __syncthreads();
  // 3. halves (A = 0..63, B = 64..127): T = L(B, A) X(A, A), X(B, A) = -X(B, B) T;
  //    thread: column tid % 64, rows 8 (tid / 64) .. + 7
  {
    const int c = tid & 63, r0 = 8 * (tid >> 6);
    smem_tile_product<8, 64>(Ls + 64 * LD, LD, X, LD, T, 65, r0, c, 1.f);
    __syncthreads();
    smem_tile_product<8, 64>(X + 64 * LD + 64, LD, T, 65, X + 64 * LD, LD, r0, c, -1.f);
  }
  __syncthreads();
}

__global__ void __launch_bounds__(4 * kMixedNB)
unit_lower_inverse_kernel(const float* __restrict__ L, int64_t ld, int nb, float* __restrict__ M, int unit)
{
  griddep_launch_dependents();
  griddep_wait();
  extern __shared__ float sm[];
  tri_inverse_smem(L, ld, nb, unit, 0, sm);
  const float(*X)[kInvLd] = reinterpret_cast<const float(*)[kInvLd]>(sm + kMixedNB * kInvLd);
  for (int e = threadIdx.x; e < kMixedNB * kMixedNB; e += blockDim.x) {
    const int r = e % kMixedNB, c = e / kMixedNB;
    M[e] = (r < nb && c < nb && r >= c) ? (r == c ? 1.f : 0.f) - X[r][c] : 0.f;
  }
}

// Inverses of the diagonal blocks (height nbk <= kMixedNB) of the n x n
// triangle at A, one CTA per block: block b of the lower (upper = 0) or upper
// (upper = 1) triangle, unit or not, inverted into out + b nbk^2, nbk x nbk
// column-major, zero beyond the block (the persistent TRSM's dinv).
// transpose_lower = 1 stores inv(L_bb)^T = inv(L_bb^T) (for solves with L^T).
__global__ void __launch_bounds__(4 * kMixedNB)
diag_block_inverse_kernel(const float* __restrict__ A, int64_t lda, int n, int nbk, int upper, int unit,
                          int transpose_lower, float* __restrict__ out)
{
  extern __shared__ float sm[];
  const int b0 = blockIdx.x * nbk, nb = min(nbk, n - b0);
  tri_inverse_smem(A + (int64_t)b0 * lda + b0, lda, nb, unit, upper, sm);
  const float(*X)[kInvLd] = reinterpret_cast<const float(*)[kInvLd]>(sm + kMixedNB * kInvLd);
  float* o = out + (int64_t)blockIdx.x * nbk * nbk;
  for (int e = threadIdx.x; e < nbk * nbk; e += blockDim.x) {
    const int r = e % nbk, c = e / nbk;
    // lower: inv(L)(r, c) = X(r, c); upper: inv(U)(r, c) = inv(U^T)(c, r) = X(c, r)
    const bool tr = upper || transpose_lower;
    o[e] = (r < nb && c < nb) ? (tr ? X[c][r] : X[r][c]) : 0.f;
  }
}

// ------------------------------------------------------------------ streamed input
// The host-buffer LU solve copies A over the host link in column chunks (one
// cudaMemcpy2DAsync per chunk, on a copy stream), so that the factorization
// starts on the first chunk while the others are still in flight: the link
// moves about 210 GB/s, which makes A's transfer 2.6 ms of a 33 ms solve at
// n = 8192.  Chunk 0 holds the first blocks.  The next chunks join the
// look-ahead schedule at a planned iteration k, on the wide stream and before
// that iteration's wide update: their FP64 columns are gathered into the FP32
// working matrix through the interchanges of blocks 0..k-1 (composed into one
// row map), then the trailing updates of blocks 0..k-1 are replayed on them in
// block order.  The last chunk, the bulk of A, rolls in instead: after the
// wide update of its landing iteration it is gathered through the
// interchanges so far, and from then on it takes every iteration's
// interchanges with the wide columns and, after each wide update, replays a
// few of the updates it missed, in block order, in the wide stream's slack.
// Once it has caught up it is part of the wide updates.  Either way the
// result is the same as with every column present from the start: an
// interchange only moves a row's values, the factored columns carry the
// interchanges of their rows the same way, and each replayed update computes
// every element from the same operands in the same order.
constexpr int kInflowMinN = 2048;              // below this the copy is short next to its fixed costs
constexpr int kInflowMaxN = (int)(kBlockMapSmemMax / (2 * sizeof(int)));   // the row map's shared memory
constexpr int kInflowFirstBlocks = 4;          // chunk 0: the first four blocks
constexpr int kInflowChunkBlocks = 8;          // chunks that join at once: eight blocks each
constexpr int kInflowRollPerIteration = 2;     // updates the rolling chunk replays after each wide update
// Planning figures, as measured at n = 8192: the link's rate and the length
// of one look-ahead iteration.
constexpr double kInflowLinkBytesPerUs = 200e3;
constexpr double kInflowIterationUs = 450.0;

struct Inflow {
  const double* host = nullptr;        // column-major n x n source, leading dimension ldh
  int64_t ldh = 0;
  double* dev = nullptr;               // its FP64 device copy (the refinement's A), leading dimension ldd
  int64_t ldd = 0;
  int chunks = 0;
  int col[kInflowMaxChunks + 1] = {};  // chunk j holds the columns [col[j], col[j + 1])
  int iter[kInflowMaxChunks] = {};     // look-ahead iteration at which chunk j joins (rolling: is gathered)
  int rolling = -1;                    // the rolling chunk (the last one), or -1
  cudaEvent_t arrived[kInflowMaxChunks] = {};
};

// Chunks and iterations for order n (n >= kInflowMinN).  A chunk whose first
// block is b must be in the wide updates by iteration b - 2: iteration b - 1's
// narrow update works on block b.  The rolling chunk, gathered at iteration
// g with blocks 0..g already applied, has replayed R (k - g) blocks when
// iteration k starts, so it is in from iteration ceil(R g / (R - 1)).
static void plan_inflow(int n, Inflow& in)
{
  const int nblk = cdiv(n, kMixedNB);
  const double bytes_per_col = sizeof(double) * (double)n;
  auto landed = [&](int col) { return col * bytes_per_col / kInflowLinkBytesPerUs; };
  const double t0 = landed(std::min(n, kInflowFirstBlocks * kMixedNB));
  // iteration k's wide update starts near t0 + (k + 1) kInflowIterationUs
  auto first_after = [&](double t) { return std::max(0, (int)std::ceil((t - t0) / kInflowIterationUs) - 1); };
  const int R = kInflowRollPerIteration;
  const int g = first_after(landed(n));
  const int ready = std::max(g + 1, cdiv((int64_t)R * g, R - 1));
  const int roll_block = ready + 2;            // the rolling chunk's first block
  in.col[0] = 0;
  in.chunks = 1;
  in.rolling = -1;
  int c = std::min(n, kInflowFirstBlocks * kMixedNB);
  const int at_once_end = roll_block + kInflowChunkBlocks <= nblk ? roll_block * kMixedNB : n;
  // at least eight blocks a chunk, and few enough chunks to leave one for the rolling chunk
  const int per = std::max(kInflowChunkBlocks, cdiv(cdiv(at_once_end - c, kMixedNB), kInflowMaxChunks - 2)) * kMixedNB;
  while (c < at_once_end) {
    in.col[in.chunks++] = c;
    c = std::min(at_once_end, c + per);
  }
  if (c < n) {                                 // the rest rolls
    in.rolling = in.chunks;
    in.col[in.chunks++] = c;
  }
  in.col[in.chunks] = n;
  in.iter[0] = 0;
  for (int j = 1; j < in.chunks; ++j) {
    if (j == in.rolling) {
      in.iter[j] = std::max(g, in.iter[j - 1]);
    } else {
      in.iter[j] = std::min(first_after(landed(in.col[j + 1])), in.col[j] / kMixedNB - 2);
    }
  }
  const int last_at_once = in.rolling >= 0 ? in.rolling - 1 : in.chunks - 1;
  for (int j = last_at_once - 1; j >= 1; --j) in.iter[j] = std::min(in.iter[j], in.iter[j + 1]);
}

// The source row of every row of [0, n) after the interchanges tr[0, i1),
// applied in order: one thread replays them on a map in shared memory (the
// transpositions staged beside it), then the map is written out whole.
__global__ void __launch_bounds__(1024)
row_source_map_kernel(const int* __restrict__ tr, int i1, int n, int* __restrict__ src)
{
  extern __shared__ int smap[];
  int* s_src = smap;            // [n]
  int* s_tr = smap + n;         // [i1]
  for (int r = threadIdx.x; r < n; r += blockDim.x) s_src[r] = r;
  for (int i = threadIdx.x; i < i1; i += blockDim.x) s_tr[i] = tr[i];
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 0; i < i1; ++i) {
      const int p = s_tr[i];
      if (p > i && p < n) {
        const int t = s_src[i];
        s_src[i] = s_src[p];
        s_src[p] = t;
      }
    }
  }
  __syncthreads();
  for (int r = threadIdx.x; r < n; r += blockDim.x) src[r] = s_src[r];
}

// out(r, c) = (float) a(src[r], c) for an m x nc block (src null: the
// identity).  Grid (row groups of 256, columns).
__global__ void __launch_bounds__(256)
gather_rows_f32_kernel(const double* __restrict__ a, int64_t lda, const int* __restrict__ src,
                       float* __restrict__ out, int64_t ldo, int m)
{
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= m) return;
  const int64_t c = blockIdx.y;
  out[c * ldo + r] = (float)a[c * lda + (src ? src[r] : r)];
}

static int block_update(cudaStream_t s, int n, float* A, int64_t lda, int k, int kb, int c0, int c1,
                        const float* minv, DeviceStatus* st, int kind, TcWorkspace& tcw, int max_ctas);

// Chunk j on stream ws (see the section comment): gathered through the
// interchanges of blocks 0..swapped-1, then the updates of blocks
// 0..replay-1 replayed on it.
static int inflow_join(cudaStream_t ws, int n, float* A, int64_t lda, const int* tr, const Inflow& in, int j,
                       int swapped, int replay, const float* minv_all, DevBuf& srcmap, DeviceStatus* st, int kind,
                       TcWorkspace& tcw, int max_ctas)
{
  const int c0 = in.col[j], nc = in.col[j + 1] - c0;
  GBS_CUDA_TRY(cudaStreamWaitEvent(ws, in.arrived[j], 0));
  const int* map = nullptr;
  const int i1 = std::min(n, swapped * kMixedNB);
  if (i1 > 0) {
    const size_t smem = sizeof(int) * ((size_t)n + i1);
    static const cudaError_t attr = cudaFuncSetAttribute(
        row_source_map_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kBlockMapSmemMax);
    GBS_CUDA_TRY(attr);
    GBS_TRY(srcmap.reserve(sizeof(int) * (size_t)n));
    PhaseScope ps(ws, PH_LASWP, 0.0, sizeof(int) * (2.0 * n + i1));
    row_source_map_kernel<<<1, 1024, smem, ws>>>(tr, i1, n, srcmap.as<int>());
    GBS_CUDA_TRY(cudaGetLastError());
    map = srcmap.as<int>();
  }
  {
    PhaseScope ps(ws, PH_COPY, 0.0, 12.0 * (double)n * nc);
    gather_rows_f32_kernel<<<dim3(cdiv(n, 256), nc), 256, 0, ws>>>(in.dev + (int64_t)c0 * in.ldd, in.ldd, map,
                                                                 A + (int64_t)c0 * lda, lda, n);
    GBS_CUDA_TRY(cudaGetLastError());
  }
  for (int b = 0; b < replay; ++b)
    GBS_TRY(block_update(ws, n, A, lda, b * kMixedNB, kMixedNB, c0, c0 + nc,
                         minv_all + (size_t)b * kMixedNB * kMixedNB, st, kind, tcw, max_ctas));
  return GBS_SUCCESS;
}

// Panels of the outer block [k, k+kb): each 32-column panel, its row
// interchanges and the block-internal update of the block's columns right of
// it.  defer: the interchanges are applied inside the block only, and the
// caller applies the whole block's interchanges to the other columns later
// (row interchanges commute with the row-wise trailing updates in between).
static int block_panels(cudaStream_t s, int n, float* A, int64_t lda, int* tr, DeviceStatus* st, DevBuf& scratch,
                        int kind, TcWorkspace& tcw, DevBuf& map, int k, int kb, bool defer, bool tournament)
{
  const int lo = defer ? k : 0, hi = defer ? k + kb : n;
  for (int j = k; j < k + kb; j += kPanelNB) {
    const int jb = std::min(kPanelNB, k + kb - j);
    float* Ajj = A + (int64_t)j * lda + j;
    const int rest = k + kb - (j + jb);
    const int* pmap = nullptr;
    bool fused = false;       // interchanges + U12 of the block's columns right of the panel done in the panel
    GBS_TRY(panel_factor<float>(s, Ajj, lda, n - j, jb, j, tr + j, scratch, st, &pmap, rest, &fused, tournament));
    if (pmap && fused) GBS_TRY(laswp_map_apply<float>(s, A, lda, pmap, lo, j, k + kb, hi));
    else if (pmap) GBS_TRY(laswp_map_apply<float>(s, A, lda, pmap, lo, j, j + jb, hi));
    else GBS_TRY(laswp_gather_device<float>(s, A, lda, tr, j, j + jb, lo, j, j + jb, hi, map));
    if (rest > 0) {
      float* A12 = A + (int64_t)(j + jb) * lda + j;
      if (!fused) {
        PhaseScope ps(s, PH_TRSM_LU, (double)jb * jb * rest, 8.0 * jb * rest);
        trsm_lunit_kernel<float, kPanelNB><<<cdiv(rest, 128), 128, 0, s>>>(Ajj, lda, jb, A12, lda, rest);
        GBS_CUDA_TRY(cudaGetLastError());
      }
      const int rows = n - (j + jb);
      if (rows > 0)
        GBS_TRY(tc_gemm_sub(s, kind, rows, rest, jb, Ajj + jb, 1, lda, A12, 1, lda, A12 + jb, lda, 0, st, tcw));
    }
  }
  return GBS_SUCCESS;
}

// I - L11^-1 of the block [k, k+kb) into minv.
static int block_inverse(cudaStream_t s, const float* A, int64_t lda, int k, int kb, float* minv)
{
  PhaseScope ps(s, PH_TRSM_LU, (double)kb * kb * kb / 3.0, sizeof(float) * 2.0 * kb * kb);
  GBS_CUDA_TRY(launch_pdl(unit_lower_inverse_kernel, dim3(1), dim3(4 * kMixedNB), kInvSmem, s,
                          (const float*)(A + (int64_t)k * lda + k), lda, kb, minv, 1));
  return GBS_SUCCESS;
}

// Trailing update of block [k, k+kb) on the columns [c0, c1):
// U12 = A12 - (I - L11^-1) A12 (the GEMM packs its operands first, so C may
// alias B), then A22 -= L21 U12.  max_ctas > 0 caps the GEMMs' persistent grid.
static int block_update(cudaStream_t s, int n, float* A, int64_t lda, int k, int kb, int c0, int c1,
                        const float* minv, DeviceStatus* st, int kind, TcWorkspace& tcw, int max_ctas)
{
  const int nc = c1 - c0, rows = n - k - kb;
  if (nc <= 0) return GBS_SUCCESS;
  float* Akk = A + (int64_t)k * lda + k;
  float* A12 = A + (int64_t)c0 * lda + k;
  GBS_TRY(tc_gemm_sub(s, kind, kb, nc, kb, minv, 1, kMixedNB, A12, 1, lda, A12, lda, 0, st, tcw, max_ctas));
  GBS_TRY(tc_gemm_sub(s, kind, rows, nc, kb, Akk + kb, 1, lda, A12, 1, lda, A12 + kb, lda, 0, st, tcw, max_ctas));
  return GBS_SUCCESS;
}

// The look-ahead schedule (la != null).  Caller's stream s, side stream ss
// (panels), wide stream ws (the caller's own without an SM partition):
//   ss: panels of block 0, I - L11^-1 of block 0
//   for each block k:
//     s:  wait for block k's panels and block k-1's wide update; block k's
//         interchanges on block k+1's columns (beside block k's I - L11^-1,
//         which follows the panels on ss)
//     ss: wait for those interchanges; update of block k+1's columns
//         (narrow); panels of block k+1, then its I - L11^-1
//     ws: wait for the narrow update; the streamed chunks that join at
//         iteration k (in != null); block k's interchanges on the other
//         columns; update of the columns right of block k+1 (wide), up to
//         the last joined chunk; then the rolling chunk's gather and replays
// The row maps and L11 inverses alternate between two buffers by block, so
// that s never rewrites one that ws may still read (with streamed input every
// block keeps its inverse, which the joins replay).  Every element sees the
// same operations in the same order as in the plain schedule, so both give
// identical factors and interchanges.
static int getrf_lookahead(cudaStream_t s, int n, float* A, int64_t lda, int* tr, DeviceStatus* st, DevBuf& scratch,
                           int kind, TcWorkspace& tcw, Lookahead& la, bool tournament, const Inflow* in)
{
  cudaStream_t ss = la.side;
  const bool split = la.wide != nullptr;
  cudaStream_t ws = split ? la.wide : s;
  const int nblk = cdiv(n, kMixedNB);
  if (in) GBS_TRY(la.minv_all.reserve(sizeof(float) * (size_t)nblk * kMixedNB * kMixedNB));
  auto minv_of = [&](int blk) -> float* {
    return in ? la.minv_all.as<float>() + (size_t)blk * kMixedNB * kMixedNB : la.minv[blk & 1].as<float>();
  };
  int joined = 1;                              // chunks in the schedule (chunk 0 from the start)
  int frontier = in ? in->col[1] : n;          // columns [0, frontier) take the wide updates
  int gathered = frontier;                     // columns [0, gathered) take the interchanges
  const int at_once = in ? (in->rolling >= 0 ? in->rolling : in->chunks) : 1;
  bool rolled_in = in == nullptr || in->rolling < 0;
  int replayed = -1;                           // blocks the rolling chunk has taken (-1: not gathered)
  // without a partition, the panel's cluster and its small kernels keep two
  // clusters' worth of SMs from the wide update's persistent grid
  auto wide_ctas = [&](int rows) {
    return split ? la.wide_sms : device_sm_count() - std::min(2 * panel_cluster_ctas(rows), device_sm_count() / 2);
  };
  GBS_CUDA_TRY(cudaEventRecord(la.ready, s));
  GBS_CUDA_TRY(cudaStreamWaitEvent(ss, la.ready, 0));
  GBS_TRY(block_panels(ss, n, A, lda, tr, st, scratch, kind, la.tc_side, la.map_side, 0, std::min(kMixedNB, n), true,
                       tournament));
  GBS_CUDA_TRY(cudaEventRecord(la.panels, ss));
  if (n > kMixedNB) GBS_TRY(block_inverse(ss, A, lda, 0, kMixedNB, minv_of(0)));
  bool wide_pending = false;
  for (int k = 0, blk = 0; k < n; k += kMixedNB, ++blk) {
    const int kb = std::min(kMixedNB, n - k);
    const int nr = n - k - kb;
    DevBuf& mapk = la.map[blk & 1];
    float* minv = minv_of(blk);
    GBS_CUDA_TRY(cudaStreamWaitEvent(s, la.panels, 0));
    if (wide_pending) GBS_CUDA_TRY(cudaStreamWaitEvent(s, la.wide_done, 0));
    if (nr == 0) {
      GBS_TRY(laswp_block_device<float>(s, A, lda, n, tr, k, k + kb, 0, k, k + kb, k + kb, mapk));
      break;
    }
    const int nb1 = std::min(kMixedNB, nr), c1 = k + kb + nb1;
    if (frontier < c1) {
      gbs_set_last_message("streamed input: a chunk joins after its columns are needed");
      return GBS_INVALID_ARGUMENT;
    }
    // the interchanges on block k+1's columns gate its panels (they run on s
    // beside block k's L11 inverse on ss); the left and wide columns get them
    // (same map) while those panels run
    GBS_TRY(laswp_block_device<float>(s, A, lda, n, tr, k, k + kb, k + kb, c1, c1, c1, mapk));
    GBS_CUDA_TRY(cudaEventRecord(la.swapped, s));
    GBS_CUDA_TRY(cudaStreamWaitEvent(ss, la.swapped, 0));
    GBS_TRY(block_update(ss, n, A, lda, k, kb, k + kb, c1, minv, st, kind, la.tc_side, 0));
    GBS_CUDA_TRY(cudaEventRecord(la.ready, ss));
    if (split) GBS_CUDA_TRY(cudaStreamWaitEvent(ws, la.ready, 0));
    GBS_TRY(block_panels(ss, n, A, lda, tr, st, scratch, kind, la.tc_side, la.map_side, k + kb, nb1, true, tournament));
    GBS_CUDA_TRY(cudaEventRecord(la.panels, ss));
    if (c1 < n) GBS_TRY(block_inverse(ss, A, lda, k + kb, nb1, minv_of(blk + 1)));
    for (; joined < at_once && in->iter[joined] <= blk; ++joined) {
      GBS_TRY(inflow_join(ws, n, A, lda, tr, *in, joined, blk, blk, la.minv_all.as<float>(), la.srcmap, st, kind,
                          split ? la.tc_wide : tcw, wide_ctas(nr)));
      frontier = gathered = in->col[joined + 1];
    }
    if (!rolled_in && replayed == blk) {       // the rolling chunk has caught up
      rolled_in = true;
      frontier = in->col[in->rolling + 1];
      joined = in->chunks;
    }
    GBS_TRY(laswp_map_apply<float>(ws, A, lda, mapk.as<int>(), 0, k, c1, std::max(c1, gathered)));
    GBS_TRY(block_update(ws, n, A, lda, k, kb, c1, frontier, minv, st, kind, split ? la.tc_wide : tcw, wide_ctas(nr)));
    if (split) {
      GBS_CUDA_TRY(cudaEventRecord(la.wide_done, ws));
      wide_pending = true;
    }
    // the rolling chunk works after the wide update's event, so that the next
    // narrow update does not wait for it
    if (!rolled_in && replayed < 0 && joined == at_once && in->iter[in->rolling] <= blk) {
      GBS_TRY(inflow_join(ws, n, A, lda, tr, *in, in->rolling, blk + 1, 0, la.minv_all.as<float>(), la.srcmap, st,
                          kind, split ? la.tc_wide : tcw, wide_ctas(nr)));
      replayed = 0;
      gathered = in->col[in->rolling + 1];
    }
    for (int q = 0; !rolled_in && replayed >= 0 && q < kInflowRollPerIteration && replayed <= blk; ++q, ++replayed)
      GBS_TRY(block_update(ws, n, A, lda, replayed * kMixedNB, kMixedNB, in->col[in->rolling], in->col[in->rolling + 1],
                           la.minv_all.as<float>() + (size_t)replayed * kMixedNB * kMixedNB, st, kind,
                           split ? la.tc_wide : tcw, wide_ctas(nr)));
  }
  if (in && (joined < in->chunks || !rolled_in)) {
    gbs_set_last_message("streamed input: a chunk never joined the schedule");
    return GBS_INVALID_ARGUMENT;
  }
  return GBS_SUCCESS;
}

int mixed_getrf(cudaStream_t s, int n, float* A, int64_t lda, int* tr, DeviceStatus* st, DevBuf& scratch, int kind,
                TcWorkspace& tcw, DevBuf& map, DevBuf& minv, Lookahead* la, bool tournament, const Inflow* in)
{
  GBS_TRY(minv.reserve(sizeof(float) * kMixedNB * kMixedNB));
  GBS_CUDA_TRY(cudaFuncSetAttribute(unit_lower_inverse_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)kInvSmem));
  GBS_CUDA_TRY(cudaFuncSetAttribute(diag_block_inverse_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)kInvSmem));
  if (la && n > kMixedNB) {
    GBS_TRY(la->init());
    const int rc = getrf_lookahead(s, n, A, lda, tr, st, scratch, kind, tcw, *la, tournament, in);
    if (rc != GBS_SUCCESS) {                    // nothing of the other streams outlives the call
      cudaStreamSynchronize(la->side);
      if (la->wide) cudaStreamSynchronize(la->wide);
    }
    return rc;
  }
  for (int k = 0; k < n; k += kMixedNB) {
    const int kb = std::min(kMixedNB, n - k);
    GBS_TRY(block_panels(s, n, A, lda, tr, st, scratch, kind, tcw, map, k, kb, false, tournament));
    if (n - k - kb > 0) {
      GBS_TRY(block_inverse(s, A, lda, k, kb, minv.as<float>()));
      GBS_TRY(block_update(s, n, A, lda, k, kb, k + kb, n, minv.as<float>(), st, kind, tcw, 0));
    }
  }
  return GBS_SUCCESS;
}

// Cholesky of the lower triangle of As (FP32, ld = lda) with the reference's
// block size; diagonal blocks and TRSM on FP32 cores, SYRK on tensor cores.
// Block k of the Cholesky: the diagonal block's factor, then
// A21 <- A21 L11^-T = A21 - A21 (I - L11^-T) (W = I - L11^-1 read transposed
// as the GEMM's B), for b <= kMixedNB.
static int potrf_block(cudaStream_t s, int n, float* As, int64_t lda, int k, int b, DeviceStatus* st, int kind,
                       TcWorkspace& tcw, float* minv)
{
  const int rs = n - k - b;
  float* Akk = As + (int64_t)k * lda + k;
  {
    PhaseScope ps(s, PH_POTRF_DIAG, (double)b * b * b / 3.0, 4.0 * b * b);
    GBS_CUDA_TRY(launch_pdl(potrf_diag_kernel<float>, dim3(1), dim3(256), potrf_diag_smem<float>(b), s, Akk, lda, b, k,
                            st));
  }
  if (rs <= 0) return GBS_SUCCESS;
  float* A21 = Akk + b;
  {
    PhaseScope ps(s, PH_TRSM_LLT, (double)b * b * b / 3.0, 8.0 * b * b);
    GBS_CUDA_TRY(launch_pdl(unit_lower_inverse_kernel, dim3(1), dim3(4 * kMixedNB), kInvSmem, s, (const float*)Akk, lda,
                            b, minv, 0));
  }
  return tc_gemm_sub(s, kind, rs, b, b, A21, 1, lda, minv, kMixedNB, 1, A21, lda, 0, st, tcw);
}

// The SYRK of block k restricted to the columns [c0, c1): the lower part of
// A(c0:n, c0:c1) -= A(c0:n, k:k+b) A(c0:c1, k:k+b)^T.
static int potrf_syrk(cudaStream_t s, int n, float* As, int64_t lda, int k, int b, int c0, int c1, DeviceStatus* st,
                      int kind, TcWorkspace& tcw, int max_ctas)
{
  if (c1 <= c0) return GBS_SUCCESS;
  const float* P = As + (int64_t)k * lda + c0;             // rows c0.. of block k's columns
  return tc_gemm_sub(s, kind, n - c0, c1 - c0, b, P, 1, lda, P, lda, 1, As + (int64_t)c0 * lda + c0, lda, 1, st,
                     tcw, max_ctas);
}

// Look-ahead Cholesky (same streams as the LU's): block k+1's diagonal
// factor and TRSM on the panel stream while the wide stream applies block k's
// SYRK to the columns right of block k+1; the caller's stream applies block
// k's SYRK to block k+1's columns in between.  Same operations per element in
// the same order as the single-stream loop.
static int potrf_lookahead(cudaStream_t s, int n, float* As, int64_t lda, int b, DeviceStatus* st, int kind,
                           TcWorkspace& tcw, Lookahead& la)
{
  cudaStream_t ss = la.side;
  const bool split = la.wide != nullptr;
  cudaStream_t ws = split ? la.wide : s;
  float* minv = la.minv[0].as<float>();
  GBS_CUDA_TRY(cudaEventRecord(la.ready, s));
  GBS_CUDA_TRY(cudaStreamWaitEvent(ss, la.ready, 0));
  GBS_TRY(potrf_block(ss, n, As, lda, 0, std::min(b, n), st, kind, la.tc_side, minv));
  GBS_CUDA_TRY(cudaEventRecord(la.panels, ss));
  bool wide_pending = false;
  for (int k = 0; k < n; k += b) {
    const int kb = std::min(b, n - k);
    const int rs = n - k - kb;
    GBS_CUDA_TRY(cudaStreamWaitEvent(s, la.panels, 0));
    if (wide_pending) GBS_CUDA_TRY(cudaStreamWaitEvent(s, la.wide_done, 0));
    if (rs == 0) break;
    const int nb1 = std::min(b, rs), c1 = k + kb + nb1;
    GBS_TRY(potrf_syrk(s, n, As, lda, k, kb, k + kb, c1, st, kind, tcw, 0));
    GBS_CUDA_TRY(cudaEventRecord(la.ready, s));
    GBS_CUDA_TRY(cudaStreamWaitEvent(ss, la.ready, 0));
    if (split) GBS_CUDA_TRY(cudaStreamWaitEvent(ws, la.ready, 0));
    GBS_TRY(potrf_block(ss, n, As, lda, k + kb, nb1, st, kind, la.tc_side, minv));
    GBS_CUDA_TRY(cudaEventRecord(la.panels, ss));
    const int ctas = split ? la.wide_sms : 0;
    GBS_TRY(potrf_syrk(ws, n, As, lda, k, kb, c1, n, st, kind, split ? la.tc_wide : tcw, ctas));
    if (split) {
      GBS_CUDA_TRY(cudaEventRecord(la.wide_done, ws));
      wide_pending = true;
    }
  }
  return GBS_SUCCESS;
}

int mixed_potrf(cudaStream_t s, int n, float* As, int64_t lda, DeviceStatus* st, int kind, TcWorkspace& tcw,
                DevBuf& minv, Lookahead* la)
{
  GBS_TRY(minv.reserve(sizeof(float) * kMixedNB * kMixedNB));
  GBS_CUDA_TRY(cudaFuncSetAttribute(unit_lower_inverse_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)kInvSmem));
  constexpr int max_bs = 128;
  static const cudaError_t attr = [] {         // once per process (thread-safe static initialisation)
    cudaError_t e = cudaFuncSetAttribute(potrf_diag_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)potrf_diag_smem<float>(max_bs));
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(trsm_rlt_kernel<float, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)(sizeof(float) * (max_bs * (max_bs + 1) + max_bs * 64 + max_bs)));
    return e;
  }();
  GBS_CUDA_TRY(attr);
  int bs = n < 32 ? n : std::min(std::max((n / 8 / 16) * 16, 8), max_bs);
  if (la && bs == kMixedNB && n > 2 * kMixedNB) {
    GBS_TRY(la->init());
    const int rc = potrf_lookahead(s, n, As, lda, bs, st, kind, tcw, *la);
    if (rc != GBS_SUCCESS) {                    // nothing of the other streams outlives the call
      cudaStreamSynchronize(la->side);
      if (la->wide) cudaStreamSynchronize(la->wide);
    }
    return rc;
  }
  for (int k = 0; k < n; k += bs) {
    const int b = std::min(bs, n - k);
    const int rs = n - k - b;
    if (b <= kMixedNB) {
      GBS_TRY(potrf_block(s, n, As, lda, k, b, st, kind, tcw, minv.as<float>()));
    } else {
      float* Akk = As + (int64_t)k * lda + k;
      {
        PhaseScope ps(s, PH_POTRF_DIAG, (double)b * b * b / 3.0, 4.0 * b * b);
        potrf_diag_kernel<float><<<1, 256, potrf_diag_smem<float>(b), s>>>(Akk, lda, b, k, st);
        GBS_CUDA_TRY(cudaGetLastError());
      }
      if (rs > 0) {
        PhaseScope ps(s, PH_TRSM_LLT, (double)rs * b * b, 8.0 * rs * b);
        trsm_rlt_kernel<float, 64><<<cdiv(rs, 64), 64, sizeof(float) * (b * (b + 1) + b * 64 + b), s>>>(
            Akk, lda, b, Akk + b, lda, rs, st);
        GBS_CUDA_TRY(cudaGetLastError());
      }
    }
    if (rs > 0) GBS_TRY(potrf_syrk(s, n, As, lda, k, b, k + b, n, st, kind, tcw, 0));
  }
  return GBS_SUCCESS;
}

// ------------------------------------------------------------------ refinement engine
struct Problem {
  int n, nrhs;
  const double* A;
  int64_t lda;
  int sym;            // 1: A symmetric, lower triangle stored
  const double* B;
  int64_t ldb;
  double* X;
  int64_t ldx;
};

// Applies M^-1 to W32 (packed n x nrhs, FP32) in place.
struct Precond {
  int kind;           // 0 = LU (A32, tr), 1 = scaled LLT (As32 lower, d32)
  int n;
  float* F;
  const int* tr;
  const float* d;
  const int* perm;    // LU: row order of P, applied when the right-hand side is converted (may be null)
  const float* dinv_l = nullptr;   // LU: inverses of the diagonal blocks of L and U for the solves (may be null)
  const float* dinv_u = nullptr;
};

// W <- M^-1 W.  LU with perm: W was gathered by perm on conversion, so only
// the two triangular solves remain.
static int precond_apply(cudaStream_t s, const Precond& M, float* W, int nrhs, SolveWork& sw)
{
  if (M.kind == 0 && M.perm) {
    GBS_TRY(tri_solve_device<float>(s, M.n, nrhs, M.F, M.n, 1, 0, 1, W, M.n, sw, M.dinv_l));
    return tri_solve_device<float>(s, M.n, nrhs, M.F, M.n, 0, 0, 0, W, M.n, sw, M.dinv_u);
  }
  if (M.kind == 0) return lu_solve_device<float>(s, M.n, nrhs, M.F, M.n, M.tr, W, M.n, 0, sw);
  const int64_t tot = (int64_t)M.n * nrhs;
  count_launch();
  diag_scale_f32_kernel<<<cdiv(tot, 256), 256, 0, s>>>(M.n, nrhs, M.d, W);
  if (M.dinv_l) {                          // L y = w, then L^T z = y, block steps with inverted diagonal blocks
    GBS_TRY(tri_solve_device<float>(s, M.n, nrhs, M.F, M.n, 1, 0, 0, W, M.n, sw, M.dinv_l));
    GBS_TRY(tri_solve_device<float>(s, M.n, nrhs, M.F, M.n, 1, 1, 0, W, M.n, sw, M.dinv_u));
  } else {
    GBS_TRY(llt_solve_device<float>(s, M.n, nrhs, M.F, M.n, 0, W, M.n, sw));
  }
  count_launch();
  diag_scale_f32_kernel<<<cdiv(tot, 256), 256, 0, s>>>(M.n, nrhs, M.d, W);
  GBS_CUDA_TRY(cudaGetLastError());
  return GBS_SUCCESS;
}

// Y = A X (B == null) or Y = B - A X, FP64 (Y with leading dimension ldy)
// Slices A for the tensor-core residuals when the options ask for them, on
// the auxiliary stream (joined by the first residual, and by AuxJoin at the
// end of the call whatever path it took).
// ready: A is complete in device memory after this event (null: after the
// work issued on s so far).
static int prepare_residual(cudaStream_t s, const Problem& P, int mode, MixedWork& w, cudaEvent_t ready = nullptr)
{
  w.oz.ready = false;
  const bool oz = mode == GBS_RESID_OZAKI || (mode == GBS_RESID_AUTO && P.n >= kOzakiMinN);
  if (!oz || P.sym) return GBS_SUCCESS;        // the residuals of a lower-stored A stay on FP64 FMA
  GBS_TRY(w.aux.fork_from(s, ready));
  w.aux.pending = true;
  const int rc = w.oz.prepare(w.aux.s, P.n, P.A, P.lda);
  GBS_CUDA_TRY(cudaEventRecord(w.aux.join, w.aux.s));
  return rc;
}

// Nothing of the auxiliary stream outlives the call that issued it.
struct AuxJoin {
  MixedWork& w;
  explicit AuxJoin(MixedWork& w_) : w(w_) {}
  ~AuxJoin()
  {
    if (w.aux.pending) cudaEventSynchronize(w.aux.join);
    w.aux.pending = false;
  }
};

static int apply_a(cudaStream_t s, const Problem& P, const double* X, int64_t ldx, const double* B, int64_t ldb, double* Y,
                   int64_t ldy, int nrhs, MixedWork& w)
{
  const int n = P.n;
  if (w.oz.ready && w.oz.n == n && nrhs <= kResRC) {
    if (w.aux.pending) {
      GBS_CUDA_TRY(cudaStreamWaitEvent(s, w.aux.join, 0));
      w.aux.pending = false;
    }
    GBS_TRY(solve_err_slot(s, w.sw));
    return ozaki_residual(s, w.oz, nrhs, X, ldx, B, ldb, Y, ldy, w.ozw, w.sw.err.as<int>());
  }
  const int splits = std::max(1, std::min(32, cdiv((int64_t)device_sm_count() * 4, cdiv(n, kResRows))));
  const int kspan = cdiv(cdiv(n, splits), kResKC) * kResKC;
  const int used = cdiv(n, kspan);
  GBS_TRY(w.part.reserve(sizeof(double) * (size_t)used * n * nrhs));
  {
    PhaseScope ps(s, PH_RESIDUAL, 2.0 * n * (double)n * nrhs, 8.0 * ((double)n * n + 2.0 * n * nrhs));
    const dim3 grid(cdiv(n, kResRows), used);
    if (nrhs <= 4) mv_partial_kernel<4><<<grid, kResRows, 0, s>>>(n, nrhs, P.A, P.lda, X, ldx, kspan, w.part.as<double>());
    else if (nrhs <= 8) mv_partial_kernel<8><<<grid, kResRows, 0, s>>>(n, nrhs, P.A, P.lda, X, ldx, kspan, w.part.as<double>());
    else mv_partial_kernel<16><<<grid, kResRows, 0, s>>>(n, nrhs, P.A, P.lda, X, ldx, kspan, w.part.as<double>());
    GBS_CUDA_TRY(cudaGetLastError());
  }
  count_launch();
  residual_reduce_kernel<<<cdiv((int64_t)n * nrhs, 256), 256, 0, s>>>(n, nrhs, used, w.part.as<double>(), B, ldb, Y,
                                                                      ldy);
  GBS_CUDA_TRY(cudaGetLastError());
  return GBS_SUCCESS;
}

// max_j backward error of the current X (computes R = B - A X into w.r)
static int backward_error(cudaStream_t s, const Problem& P, double anorm, MixedWork& w, double* be)
{
  const int n = P.n, nrhs = P.nrhs;
  double* R = w.r.as<double>();
  GBS_TRY(apply_a(s, P, P.X, P.ldx, P.B, P.ldb, R, n, nrhs, w));
  count_launch();
  col_absmax3_kernel<<<dim3(nrhs, 3), 256, 0, s>>>(n, nrhs, R, n, P.X, P.ldx, P.B, P.ldb, w.stats.as<double>());
  GBS_CUDA_TRY(cudaGetLastError());
  double* h = (double*)w.hstats.p;
  GBS_CUDA_TRY(cudaMemcpyAsync(h, w.stats.p, sizeof(double) * 3 * nrhs, cudaMemcpyDeviceToHost, s));
  GBS_TRY(solve_status(s, w.sw));
  double worst = 0.0;
  for (int c = 0; c < nrhs; ++c) {
    const double den = anorm * h[nrhs + c] + h[2 * nrhs + c];
    double e = den > 0 ? h[c] / den : h[c];
    if (e != e) e = INFINITY;
    worst = std::max(worst, e);
  }
  *be = worst;
  return GBS_SUCCESS;
}

// D64 (n x nrhs, ld n) = M^-1 Y64 via FP32 with per-column scaling
static int precond_f64(cudaStream_t s, const Precond& M, const double* Y, double* D, int nrhs, MixedWork& w)
{
  const int n = M.n;
  const int64_t tot = (int64_t)n * nrhs;
  double* sc = w.stats.as<double>() + 3 * nrhs;
  count_launch();
  col_absmax3_kernel<<<dim3(nrhs, 1), 256, 0, s>>>(n, nrhs, Y, n, Y, n, Y, n, sc);
  count_launch();
  scale_to_f32_kernel<<<cdiv(tot, 256), 256, 0, s>>>(n, nrhs, Y, n, sc, w.w32.as<float>(), M.perm);
  GBS_CUDA_TRY(cudaGetLastError());
  GBS_TRY(precond_apply(s, M, w.w32.as<float>(), nrhs, w.sw));
  count_launch();
  update_from_f32_kernel<<<cdiv(tot, 256), 256, 0, s>>>(n, nrhs, w.w32.as<float>(), sc, D, n, 1);
  GBS_CUDA_TRY(cudaGetLastError());
  return GBS_SUCCESS;
}

// One GMRES-IR correction: X += d with (M^-1 A) d ~= M^-1 r (r = w.r).
static int gmres_correction(cudaStream_t s, const Problem& P, const Precond& M, int mmax, double tau, MixedWork& w,
                            int* inner_its)
{
  const int n = P.n, nrhs = P.nrhs;
  const int64_t slab = (int64_t)n * nrhs;
  GBS_TRY(w.v.reserve(sizeof(double) * (size_t)slab * (mmax + 1)));
  GBS_TRY(w.z.reserve(sizeof(double) * (size_t)slab));
  GBS_TRY(w.coef.reserve(sizeof(double) * (size_t)(mmax + 2) * nrhs * 2));
  double* V = w.v.as<double>();
  double* Z = w.z.as<double>();
  double* coef = w.coef.as<double>();
  std::vector<double> hcoef((size_t)(mmax + 2) * nrhs);
  // z0 = M^-1 r ; beta = ||z0|| ; V_0 = z0 / beta
  GBS_TRY(precond_f64(s, M, w.r.as<double>(), Z, nrhs, w));
  count_launch();
  gmres_dots_kernel<<<dim3(1, nrhs), 256, 0, s>>>(n, nrhs, Z, Z, coef);
  GBS_CUDA_TRY(cudaMemcpyAsync(hcoef.data(), coef, sizeof(double) * nrhs, cudaMemcpyDeviceToHost, s));
  GBS_CUDA_TRY(cudaStreamSynchronize(s));
  std::vector<double> beta(nrhs), inv(nrhs);
  for (int c = 0; c < nrhs; ++c) {
    beta[c] = std::sqrt(hcoef[c]);
    inv[c] = beta[c] > 0 ? 1.0 / beta[c] : 0.0;
  }
  GBS_CUDA_TRY(cudaMemcpyAsync(coef, inv.data(), sizeof(double) * nrhs, cudaMemcpyHostToDevice, s));
  count_launch();
  gmres_scale_kernel<<<cdiv(slab, 256), 256, 0, s>>>(n, nrhs, Z, coef, V);
  // Hessenberg + Givens per column
  std::vector<double> H((size_t)(mmax + 1) * mmax * nrhs, 0.0), cs((size_t)mmax * nrhs), sn((size_t)mmax * nrhs),
      g((size_t)(mmax + 1) * nrhs, 0.0);
  auto Hc = [&](int i, int j, int c) -> double& { return H[((size_t)c * (mmax + 1) + i) * mmax + j]; };
  for (int c = 0; c < nrhs; ++c) g[(size_t)c * (mmax + 1)] = beta[c];
  std::vector<char> done(nrhs, 0);
  for (int c = 0; c < nrhs; ++c) done[c] = beta[c] == 0.0;
  int m = 0;
  for (int j = 0; j < mmax; ++j) {
    double* Vj = V + (int64_t)j * slab;
    double* Vn = V + (int64_t)(j + 1) * slab;
    // w = M^-1 A V_j  (into Vn as scratch)
    GBS_TRY(apply_a(s, P, Vj, n, nullptr, 0, Vn, n, nrhs, w));
    GBS_TRY(precond_f64(s, M, Vn, Z, nrhs, w));
    // CGS2: h = V^T z ; z -= V h ; twice
    std::vector<double> hsum((size_t)(j + 1) * nrhs, 0.0);
    for (int pass = 0; pass < 2; ++pass) {
      count_launch();
      gmres_dots_kernel<<<dim3(j + 1, nrhs), 256, 0, s>>>(n, nrhs, V, Z, coef);
      count_launch();
      gmres_combine_kernel<<<cdiv(slab, 256), 256, 0, s>>>(n, nrhs, j + 1, V, coef, -1.0, Z, n);
      GBS_CUDA_TRY(cudaMemcpyAsync(hcoef.data(), coef, sizeof(double) * (j + 1) * nrhs, cudaMemcpyDeviceToHost, s));
      GBS_CUDA_TRY(cudaStreamSynchronize(s));
      for (size_t q = 0; q < hsum.size(); ++q) hsum[q] += hcoef[q];
    }
    count_launch();
    gmres_dots_kernel<<<dim3(1, nrhs), 256, 0, s>>>(n, nrhs, Z, Z, coef);
    GBS_CUDA_TRY(cudaMemcpyAsync(hcoef.data(), coef, sizeof(double) * nrhs, cudaMemcpyDeviceToHost, s));
    GBS_CUDA_TRY(cudaStreamSynchronize(s));
    bool all_done = true;
    for (int c = 0; c < nrhs; ++c) {
      const double hn = std::sqrt(std::max(hcoef[c], 0.0));
      for (int i = 0; i <= j; ++i) Hc(i, j, c) = hsum[(size_t)i * nrhs + c];
      Hc(j + 1, j, c) = hn;
      inv[c] = hn > 0 ? 1.0 / hn : 0.0;
      // apply previous rotations, then a new one
      for (int i = 0; i < j; ++i) {
        const double a = Hc(i, j, c), b = Hc(i + 1, j, c);
        const double C = cs[(size_t)c * mmax + i], S = sn[(size_t)c * mmax + i];
        Hc(i, j, c) = C * a + S * b;
        Hc(i + 1, j, c) = -S * a + C * b;
      }
      const double a = Hc(j, j, c), b = Hc(j + 1, j, c);
      const double r = std::hypot(a, b);
      const double C = r > 0 ? a / r : 1.0, S = r > 0 ? b / r : 0.0;
      cs[(size_t)c * mmax + j] = C;
      sn[(size_t)c * mmax + j] = S;
      Hc(j, j, c) = r;
      Hc(j + 1, j, c) = 0.0;
      double& gj = g[(size_t)c * (mmax + 1) + j];
      double& gj1 = g[(size_t)c * (mmax + 1) + j + 1];
      gj1 = -S * gj;
      gj = C * gj;
      if (done[c] || beta[c] == 0.0 || std::fabs(gj1) <= tau * beta[c] || hn == 0.0) done[c] = 1;
      all_done = all_done && done[c];
    }
    GBS_CUDA_TRY(cudaMemcpyAsync(coef, inv.data(), sizeof(double) * nrhs, cudaMemcpyHostToDevice, s));
    count_launch();
    gmres_scale_kernel<<<cdiv(slab, 256), 256, 0, s>>>(n, nrhs, Z, coef, Vn);
    m = j + 1;
    if (all_done) break;
  }
  // y = R^-1 g (per column), X += V y
  std::vector<double> y((size_t)m * nrhs, 0.0);
  for (int c = 0; c < nrhs; ++c) {
    if (beta[c] == 0.0) continue;
    for (int i = m - 1; i >= 0; --i) {
      double acc = g[(size_t)c * (mmax + 1) + i];
      for (int k = i + 1; k < m; ++k) acc -= Hc(i, k, c) * y[(size_t)k * nrhs + c];
      const double d = Hc(i, i, c);
      y[(size_t)i * nrhs + c] = d != 0 ? acc / d : 0.0;
    }
  }
  GBS_CUDA_TRY(cudaMemcpyAsync(coef, y.data(), sizeof(double) * m * nrhs, cudaMemcpyHostToDevice, s));
  count_launch();
  gmres_combine_kernel<<<cdiv(slab, 256), 256, 0, s>>>(n, nrhs, m, V, coef, 1.0, P.X, P.ldx);
  GBS_CUDA_TRY(cudaGetLastError());
  *inner_its += m;
  return GBS_SUCCESS;
}

// Refines P.X (already holding x0) to the backward-error bound.  Returns
// converged through *ok.
static int refine(cudaStream_t s, const Problem& P, const Precond& M, bool use_gmres, const MixedOptions& opt,
                  double anorm, MixedWork& w, MixedResult& out, bool* ok)
{
  const int n = P.n, nrhs = P.nrhs;
  *ok = false;
  double prev = INFINITY;
  int stalls = 0;
  for (int it = 0; it <= opt.max_iter; ++it) {
    double be = 0;
    GBS_TRY(backward_error(s, P, anorm, w, &be));
    out.backward_error = be;
    out.iterations = it;
    if (be <= opt.tol) { *ok = true; return GBS_SUCCESS; }
    if (!(be < 0.5 * prev)) { if (++stalls >= 2) return GBS_SUCCESS; } else stalls = 0;
    prev = std::min(prev, be);
    if (it == opt.max_iter) break;
    if (use_gmres) {
      GBS_TRY(gmres_correction(s, P, M, opt.gmres_restart, opt.gmres_tol, w, &out.inner_iterations));
    } else {
      double* sc = w.stats.as<double>();
      const int64_t tot = (int64_t)n * nrhs;
      count_launch();
      scale_to_f32_kernel<<<cdiv(tot, 256), 256, 0, s>>>(n, nrhs, w.r.as<double>(), n, sc, w.w32.as<float>(),
                                                          M.perm);
      GBS_CUDA_TRY(cudaGetLastError());
      GBS_TRY(precond_apply(s, M, w.w32.as<float>(), nrhs, w.sw));
      count_launch();
      update_from_f32_kernel<<<cdiv(tot, 256), 256, 0, s>>>(n, nrhs, w.w32.as<float>(), sc, P.X, P.ldx, 0);
      GBS_CUDA_TRY(cudaGetLastError());
    }
  }
  return GBS_SUCCESS;
}

static int reserve_common(MixedWork& w, int n, int nrhs)
{
  GBS_TRY(w.st.reserve(sizeof(DeviceStatus)));
  GBS_TRY(w.r.reserve(sizeof(double) * (size_t)n * nrhs));
  GBS_TRY(w.w32.reserve(sizeof(float) * (size_t)n * nrhs));
  GBS_TRY(w.stats.reserve(sizeof(double) * (4 * nrhs + 4)));
  GBS_TRY(w.rows.reserve(sizeof(double) * (size_t)n));
  GBS_TRY(w.hstats.reserve(sizeof(double) * (4 * nrhs + 4)));
  return GBS_SUCCESS;
}

// ||A||_inf in two steps, so that the factorization is issued without waiting
// for it: norm_start puts the row sums on stream s (the auxiliary stream for
// the LU, beside the factorization) with their copy to pinned host memory;
// norm_wait waits for that copy and takes the maximum.
static int norm_start(cudaStream_t s, const Problem& P, MixedWork& w)
{
  const int rblocks = cdiv(P.n, 256);
  const int splits = P.sym ? 1 : std::max(1, std::min(cdiv(P.n, 64), 4 * device_sm_count() / rblocks));
  if (splits == 1) {
    count_launch();
    row_abs_sum_kernel<<<rblocks, 256, 0, s>>>(P.n, P.A, P.lda, P.sym, w.rows.as<double>());
  } else {
    const int kspan = cdiv(P.n, splits);
    const int used = cdiv(P.n, kspan);
    GBS_TRY(w.npart.reserve(sizeof(double) * (size_t)used * P.n));
    count_launch();
    row_abs_partial_kernel<<<dim3(rblocks, used), 256, 0, s>>>(P.n, P.A, P.lda, kspan, w.npart.as<double>());
    count_launch();
    row_abs_reduce_kernel<<<rblocks, 256, 0, s>>>(P.n, used, w.npart.as<double>(), w.rows.as<double>());
  }
  GBS_CUDA_TRY(cudaGetLastError());
  GBS_TRY(w.aux.init());
  GBS_TRY(w.hrows.reserve(sizeof(double) * (size_t)P.n));
  GBS_CUDA_TRY(cudaMemcpyAsync(w.hrows.p, w.rows.p, sizeof(double) * P.n, cudaMemcpyDeviceToHost, s));
  GBS_CUDA_TRY(cudaEventRecord(w.aux.norm, s));
  return GBS_SUCCESS;
}

static int norm_wait(MixedWork& w, int n, double* anorm)
{
  GBS_CUDA_TRY(cudaEventSynchronize(w.aux.norm));
  const double* h = static_cast<const double*>(w.hrows.p);
  double a = 0;
  for (int i = 0; i < n; ++i) a = std::max(a, h[i]);
  *anorm = a;
  return GBS_SUCCESS;
}

static int inf_norm(cudaStream_t s, const Problem& P, MixedWork& w, double* anorm)
{
  GBS_TRY(norm_start(s, P, w));
  return norm_wait(w, P.n, anorm);
}

// x0 = M^-1 b
static int initial_solve(cudaStream_t s, const Problem& P, const Precond& M, MixedWork& w)
{
  const int n = P.n, nrhs = P.nrhs;
  const int64_t tot = (int64_t)n * nrhs;
  double* sc = w.stats.as<double>();
  count_launch();
  col_absmax3_kernel<<<dim3(nrhs, 1), 256, 0, s>>>(n, nrhs, P.B, P.ldb, P.B, P.ldb, P.B, P.ldb, sc);
  count_launch();
  scale_to_f32_kernel<<<cdiv(tot, 256), 256, 0, s>>>(n, nrhs, P.B, P.ldb, sc, w.w32.as<float>(), M.perm);
  GBS_CUDA_TRY(cudaGetLastError());
  GBS_TRY(precond_apply(s, M, w.w32.as<float>(), nrhs, w.sw));
  count_launch();
  update_from_f32_kernel<<<cdiv(tot, 256), 256, 0, s>>>(n, nrhs, w.w32.as<float>(), sc, P.X, P.ldx, 1);
  GBS_CUDA_TRY(cudaGetLastError());
  return GBS_SUCCESS;
}

template <typename Fn>
static int per_group(int nrhs, MixedResult* res, Fn fn)
{
  MixedResult worst;
  bool first = true;
  for (int c0 = 0; c0 < nrhs; c0 += kResRC) {
    MixedResult r;
    GBS_TRY(fn(c0, std::min(kResRC, nrhs - c0), &r));
    if (first) { worst = r; first = false; continue; }
    worst.iterations = std::max(worst.iterations, r.iterations);
    worst.inner_iterations = std::max(worst.inner_iterations, r.inner_iterations);
    worst.fell_back |= r.fell_back;
    worst.singular |= r.singular;
    worst.backward_error = std::max(worst.backward_error, r.backward_error);
    if (r.fell_back) worst.tier = r.tier;
  }
  if (res) *res = worst;
  return GBS_SUCCESS;
}

// ------------------------------------------------------------------ LU front end
// Nothing of the copy stream outlives the call that issued it.
struct CopyJoin {
  cudaStream_t s;
  explicit CopyJoin(cudaStream_t s_) : s(s_) {}
  ~CopyJoin()
  {
    if (s) cudaStreamSynchronize(s);
  }
};

// in != null: A (n x n, ld lda) is filled from the host by the streamed
// input, and in->dev == A.
static int lu_solve_impl(cudaStream_t s, int n, int nrhs, const double* A, int64_t lda, const double* B, int64_t ldb,
                         double* X, int64_t ldx, const MixedOptions& opt, MixedResult* res, Inflow* in)
{
  MixedResult out;
  out.tier = opt.tier;
  if (n <= 0 || nrhs <= 0) {
    if (res) *res = out;
    return GBS_SUCCESS;
  }
  if (nrhs > kResRC) {
    if (in) return GBS_INVALID_ARGUMENT;       // streamed input carries at most one group
    return per_group(nrhs, res, [&](int c0, int nc, MixedResult* r) {
      return mixed_lu_solve(s, n, nc, A, lda, B + (int64_t)c0 * ldb, ldb, X + (int64_t)c0 * ldx, ldx, opt, r);
    });
  }
  MixedLease lease;
  if (lease.status != GBS_SUCCESS) return lease.status;
  MixedWork& w = *lease.w;
  GBS_TRY(reserve_common(w, n, nrhs));
  GBS_TRY(w.a32.reserve(sizeof(float) * (size_t)n * n));
  GBS_TRY(w.tr.reserve(sizeof(int) * (size_t)n));
  DeviceStatus* st = w.st.as<DeviceStatus>();
  Problem P{n, nrhs, A, lda, 0, B, ldb, X, ldx};
  cudaEvent_t complete = nullptr;              // A is whole in device memory after this event (null: on entry)
  if (in) GBS_TRY(w.copy.init());
  CopyJoin copy_join(in ? w.copy.s : nullptr);
  if (in) {
    for (int j = 0; j < in->chunks; ++j) {
      const int c0 = in->col[j], nc = in->col[j + 1] - c0;
      GBS_CUDA_TRY(cudaMemcpy2DAsync(in->dev + (int64_t)c0 * in->ldd, sizeof(double) * in->ldd,
                                     in->host + (int64_t)c0 * in->ldh, sizeof(double) * in->ldh, sizeof(double) * n,
                                     nc, cudaMemcpyHostToDevice, w.copy.s));
      in->arrived[j] = w.copy.ev[j];
      GBS_CUDA_TRY(cudaEventRecord(in->arrived[j], w.copy.s));
    }
    complete = in->arrived[in->chunks - 1];
    GBS_CUDA_TRY(cudaStreamWaitEvent(s, in->arrived[0], 0));
  }
  // ||A||_inf and A's digit slices on the auxiliary stream, beside the factorization
  AuxJoin aux_join(w);
  GBS_TRY(w.aux.fork_from(s, complete));
  GBS_TRY(norm_start(w.aux.s, P, w));
  GBS_CUDA_TRY(cudaEventRecord(w.aux.join, w.aux.s));
  w.aux.pending = true;
  GBS_TRY(prepare_residual(s, P, opt.residual, w, complete));
  double anorm = -1;
  auto need_anorm = [&]() -> int { return anorm < 0 ? norm_wait(w, n, &anorm) : GBS_SUCCESS; };
  bool converged = false;
  if (opt.tier != GBS_TIER_FP64) {
    GBS_TRY(reset_status(st, s));
    {
      const int nc = in ? in->col[1] : n;      // streamed input: the later chunks join inside the factorization
      PhaseScope ps(s, PH_COPY, 0.0, 12.0 * (double)n * nc);
      copy_matrix_kernel<double, float><<<std::min<int64_t>(cdiv((int64_t)n * nc, 256), 65535 * 8), 256, 0, s>>>(
          A, lda, w.a32.as<float>(), n, n, nc);
      GBS_CUDA_TRY(cudaGetLastError());
    }
    GBS_TRY(mixed_getrf(s, n, w.a32.as<float>(), n, w.tr.as<int>(), st, w.scratch, tc_kind(opt.tier), w.tc, w.map,
                        w.minv, opt.lookahead ? &w.la : nullptr,
                        opt.pivoting == GBS_PIVOT_TOURNAMENT, in));
    if (complete) GBS_CUDA_TRY(cudaStreamWaitEvent(s, complete, 0));
    DeviceStatus h;
    GBS_TRY(read_status(st, &h, s));
    if (h.info < 0) {
      const int* perm = nullptr;
      if (n <= kPermSmemMax) {
        GBS_TRY(w.perm.reserve(sizeof(int) * (size_t)n));
        GBS_CUDA_TRY(cudaFuncSetAttribute(perm_from_transpositions_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)(sizeof(int) * kPermSmemMax)));
        PhaseScope ps(s, PH_LASWP, 0.0, 8.0 * n);
        perm_from_transpositions_kernel<<<1, 1024, sizeof(int) * n, s>>>(n, w.tr.as<int>(), w.perm.as<int>());
        GBS_CUDA_TRY(cudaGetLastError());
        perm = w.perm.as<int>();
      }
      Precond M{0, n, w.a32.as<float>(), w.tr.as<int>(), nullptr, perm};
      if (opt.tier == GBS_TIER_TF32X3) {
        // inverses of the diagonal blocks of L and U: each correction's block step becomes a product
        // (FP32-accurate factors only: the 16-bit tiers' blocks are left to substitution)
        constexpr int nbk = tri_solve_nb<float>();
        const int nblk = (n + nbk - 1) / nbk;
        GBS_TRY(w.dinv.reserve(sizeof(float) * 2 * (size_t)nblk * nbk * nbk));
        float* dl = w.dinv.as<float>();
        float* du = dl + (size_t)nblk * nbk * nbk;
        PhaseScope ps(s, PH_TRI_SOLVE, 2.0 * nblk * nbk * nbk * nbk / 3.0, 16.0 * nblk * nbk * nbk);
        diag_block_inverse_kernel<<<nblk, 4 * kMixedNB, kInvSmem, s>>>(w.a32.as<float>(), n, n, nbk, 0, 1, 0, dl);
        diag_block_inverse_kernel<<<nblk, 4 * kMixedNB, kInvSmem, s>>>(w.a32.as<float>(), n, n, nbk, 1, 0, 0, du);
        GBS_CUDA_TRY(cudaGetLastError());
        M.dinv_l = dl;
        M.dinv_u = du;
      }
      GBS_TRY(initial_solve(s, P, M, w));
      const bool gm = opt.refine == GBS_REFINE_GMRES || (opt.refine == GBS_REFINE_AUTO && opt.tier != GBS_TIER_TF32X3);
      out.solver = gm ? GBS_REFINE_GMRES : GBS_REFINE_CLASSIC;
      GBS_TRY(need_anorm());
      GBS_TRY(refine(s, P, M, gm, opt, anorm, w, out, &converged));
    }
  }
  if (!converged) {
    out.fell_back = opt.tier != GBS_TIER_FP64;
    out.tier = GBS_TIER_FP64;
    if (complete) GBS_CUDA_TRY(cudaStreamWaitEvent(s, complete, 0));
    GBS_TRY(w.a64.reserve(sizeof(double) * (size_t)n * n));
    GBS_TRY(copy_matrix_device<double>(s, A, lda, w.a64.as<double>(), n, n, n));
    GBS_TRY(reset_status(st, s));
    GBS_TRY(getrf_device<double>(s, n, n, w.a64.as<double>(), n, w.tr.as<int>(), st, w.scratch));
    DeviceStatus h;
    GBS_TRY(read_status(st, &h, s));
    GBS_TRY(copy_matrix_device<double>(s, B, ldb, X, ldx, n, nrhs));
    GBS_TRY(lu_solve_device<double>(s, n, nrhs, w.a64.as<double>(), n, w.tr.as<int>(), X, ldx, 0, w.sw));
    GBS_TRY(need_anorm());
    GBS_TRY(backward_error(s, P, anorm, w, &out.backward_error));
    if (h.info >= 0) out.singular = 1;
  }
  if (res) *res = out;
  return GBS_SUCCESS;
}

int streamed_input_plan(int n, int cap, int* col, int* iter, int* rolling)
{
  if (n < kInflowMinN || n > kInflowMaxN) return 0;
  Inflow in;
  plan_inflow(n, in);
  for (int j = 0; j <= in.chunks && j <= cap; ++j) {
    if (col) col[j] = in.col[j];
    if (iter && j < in.chunks && j < cap) iter[j] = in.iter[j];
  }
  if (rolling) *rolling = in.rolling;
  return in.chunks;
}

int mixed_lu_solve(cudaStream_t s, int n, int nrhs, const double* A, int64_t lda, const double* B, int64_t ldb,
                   double* X, int64_t ldx, const MixedOptions& opt, MixedResult* res)
{
  return lu_solve_impl(s, n, nrhs, A, lda, B, ldb, X, ldx, opt, res, nullptr);
}

int mixed_lu_solve_host(cudaStream_t s, int n, int nrhs, const double* a, int64_t lda, double* dA, const double* B,
                        int64_t ldb, double* X, int64_t ldx, const MixedOptions& opt, MixedResult* res)
{
  const bool streamed = n >= kInflowMinN && n <= kInflowMaxN && nrhs <= kResRC && opt.tier != GBS_TIER_FP64 &&
                        opt.lookahead;
  if (!streamed) {
    GBS_CUDA_TRY(cudaMemcpy2DAsync(dA, sizeof(double) * n, a, sizeof(double) * lda, sizeof(double) * n, n,
                                   cudaMemcpyHostToDevice, s));
    return lu_solve_impl(s, n, nrhs, dA, n, B, ldb, X, ldx, opt, res, nullptr);
  }
  Inflow in;
  in.host = a;
  in.ldh = lda;
  in.dev = dA;
  in.ldd = n;
  plan_inflow(n, in);
  return lu_solve_impl(s, n, nrhs, dA, n, B, ldb, X, ldx, opt, res, &in);
}

int residual_device(cudaStream_t s, int n, int nrhs, const double* A, int64_t lda, const double* X, int64_t ldx,
                    const double* B, int64_t ldb, double* R, int64_t ldr, int method)
{
  if (n <= 0 || nrhs <= 0) return GBS_SUCCESS;
  MixedLease lease;
  if (lease.status != GBS_SUCCESS) return lease.status;
  MixedWork& w = *lease.w;
  Problem P{n, nrhs, A, lda, 0, B, ldb, nullptr, 0};
  AuxJoin aux_join(w);
  GBS_TRY(prepare_residual(s, P, method, w));
  for (int c0 = 0; c0 < nrhs; c0 += kResRC) {
    const int nc = std::min(kResRC, nrhs - c0);
    GBS_TRY(apply_a(s, P, X + (int64_t)c0 * ldx, ldx, B ? B + (int64_t)c0 * ldb : nullptr, ldb, R + (int64_t)c0 * ldr,
                    ldr, nc, w));
  }
  return solve_status(s, w.sw);
}

// ------------------------------------------------------------------ LLT front end
int mixed_llt_solve(cudaStream_t s, int n, int nrhs, const double* A, int64_t lda, const double* B, int64_t ldb,
                    double* X, int64_t ldx, const MixedOptions& opt, MixedResult* res)
{
  MixedResult out;
  out.tier = opt.tier;
  if (n <= 0 || nrhs <= 0) {
    if (res) *res = out;
    return GBS_SUCCESS;
  }
  if (nrhs > kResRC)
    return per_group(nrhs, res, [&](int c0, int nc, MixedResult* r) {
      return mixed_llt_solve(s, n, nc, A, lda, B + (int64_t)c0 * ldb, ldb, X + (int64_t)c0 * ldx, ldx, opt, r);
    });
  MixedLease lease;
  if (lease.status != GBS_SUCCESS) return lease.status;
  MixedWork& w = *lease.w;
  GBS_TRY(reserve_common(w, n, nrhs));
  GBS_TRY(w.a32.reserve(sizeof(float) * (size_t)n * n));
  GBS_TRY(w.d32.reserve(sizeof(float) * (size_t)n));
  GBS_TRY(w.d64.reserve(sizeof(double) * (size_t)n));
  GBS_TRY(w.afull.reserve(sizeof(double) * (size_t)n * n));
  DeviceStatus* st = w.st.as<DeviceStatus>();
  // the residuals read a full symmetric copy (coalesced, general kernel)
  {
    PhaseScope ps(s, PH_COPY, 0.0, 16.0 * (double)n * n);
    symmetrize_kernel<<<dim3(cdiv(n, 32), cdiv(n, 32)), dim3(32, 8), 0, s>>>(n, A, lda, w.afull.as<double>());
    spd_diag_kernel<<<cdiv(n, 256), 256, 0, s>>>(n, A, lda, w.d64.as<double>(), w.d32.as<float>());
    GBS_CUDA_TRY(cudaGetLastError());
    count_launch();
  }
  Problem P{n, nrhs, w.afull.as<double>(), n, 0, B, ldb, X, ldx};
  double anorm = 0;
  GBS_TRY(inf_norm(s, P, w, &anorm));
  AuxJoin aux_join(w);
  GBS_TRY(prepare_residual(s, P, opt.residual, w));
  bool converged = false;
  int not_spd = 0;
  if (opt.tier != GBS_TIER_FP64) {
    // unit roundoff of the factorization's products: the shift that keeps the
    // low-precision Cholesky of D A D positive (Higham & Pranesh) grows by 10
    // on each breakdown, starting at 0 for the FP32-accurate tier
    const double uf = opt.tier == GBS_TIER_BF16 ? 0x1p-8 : (opt.tier == GBS_TIER_TF32X3 ? 0x1p-24 : 0x1p-11);
    double sigma = opt.tier == GBS_TIER_TF32X3 ? 0.0 : opt.shift_factor * uf;
    for (int attempt = 0; attempt < 4 && !converged; ++attempt) {
      GBS_TRY(reset_status(st, s));
      {
        PhaseScope ps(s, PH_COPY, 0.0, 12.0 * (double)n * n);
        scale_spd_kernel<<<cdiv((int64_t)n * n, 256), 256, 0, s>>>(n, A, lda, sigma, w.d64.as<double>(),
                                                                   w.a32.as<float>());
        GBS_CUDA_TRY(cudaGetLastError());
      }
      GBS_TRY(mixed_potrf(s, n, w.a32.as<float>(), n, st, tc_kind(opt.tier), w.tc, w.minv,
                          opt.lookahead ? &w.la : nullptr));
      DeviceStatus h;
      GBS_TRY(read_status(st, &h, s));
      out.shift = sigma;
      if (h.info >= 0) {
        sigma = sigma > 0 ? sigma * 10.0 : 8.0 * uf;
        continue;
      }
      Precond M{1, n, w.a32.as<float>(), nullptr, w.d32.as<float>(), nullptr};
      if (opt.tier == GBS_TIER_TF32X3) {
        constexpr int nbk = tri_solve_nb<float>();
        const int nblk = (n + nbk - 1) / nbk;
        GBS_TRY(w.dinv.reserve(sizeof(float) * 2 * (size_t)nblk * nbk * nbk));
        float* dl = w.dinv.as<float>();
        float* dlt = dl + (size_t)nblk * nbk * nbk;
        GBS_CUDA_TRY(cudaFuncSetAttribute(diag_block_inverse_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)kInvSmem));
        PhaseScope ps(s, PH_TRI_SOLVE, 2.0 * nblk * nbk * nbk * nbk / 3.0, 16.0 * nblk * nbk * nbk);
        diag_block_inverse_kernel<<<nblk, 4 * kMixedNB, kInvSmem, s>>>(w.a32.as<float>(), n, n, nbk, 0, 0, 0, dl);
        diag_block_inverse_kernel<<<nblk, 4 * kMixedNB, kInvSmem, s>>>(w.a32.as<float>(), n, n, nbk, 0, 0, 1, dlt);
        GBS_CUDA_TRY(cudaGetLastError());
        M.dinv_l = dl;
        M.dinv_u = dlt;
      }
      GBS_TRY(initial_solve(s, P, M, w));
      const bool gm = opt.refine == GBS_REFINE_GMRES || (opt.refine == GBS_REFINE_AUTO && opt.tier != GBS_TIER_TF32X3);
      out.solver = gm ? GBS_REFINE_GMRES : GBS_REFINE_CLASSIC;
      GBS_TRY(refine(s, P, M, gm, opt, anorm, w, out, &converged));
      break;
    }
  }
  if (!converged) {
    out.fell_back = opt.tier != GBS_TIER_FP64;
    out.tier = GBS_TIER_FP64;
    GBS_TRY(w.a64.reserve(sizeof(double) * (size_t)n * n));
    GBS_TRY(copy_matrix_device<double>(s, A, lda, w.a64.as<double>(), n, n, n));
    GBS_TRY(reset_status(st, s));
    GBS_TRY(potrf_device<double>(s, n, w.a64.as<double>(), n, 0, st, w.scratch));
    DeviceStatus h;
    GBS_TRY(read_status(st, &h, s));
    if (h.info >= 0) {
      not_spd = 1;
    } else {
      GBS_TRY(copy_matrix_device<double>(s, B, ldb, X, ldx, n, nrhs));
      GBS_TRY(llt_solve_device<double>(s, n, nrhs, w.a64.as<double>(), n, 0, X, ldx, w.sw));
      GBS_TRY(backward_error(s, P, anorm, w, &out.backward_error));
    }
  }
  out.singular = not_spd;
  if (res) *res = out;
  return not_spd ? GBS_NUMERICAL_ISSUE : GBS_SUCCESS;
}

}  // namespace gbs
