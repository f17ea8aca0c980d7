// Kernels of the plain (FP64 / FP32) factor-and-solve path.  All matrices are
// column-major with a leading dimension, as the reference stores them.
//
//   panel_lu_kernel      unblocked partial-pivoting LU of an m x NB panel
//                        (PartialPivLU.h:365-409): rows live in registers, pivot
//                        search is a warp-shuffle argmax + a grid-wide reduction
//   laswp_kernel         row interchanges on column ranges (PartialPivLU.h:477-487)
//   trsm_lunit_kernel    A12 <- L11^{-1} A12, unit lower (PartialPivLU.h:490)
//   gemm_sub_kernel      C -= op(A) op(B), optional lower-triangle-only mode for
//                        SYRK (PartialPivLU.h:492, LLT.h:357)
//   potrf_diag_kernel    Cholesky of one diagonal block (LLT.h:305-328), right-looking in smem
//   trsm_rlt_kernel      A21 <- A21 L11^{-T} (LLT.h:356); trsm_rlt_blocked_kernel
//                        the same in 16-column blocks (the plain path's latency)
//   trsm_persistent_kernel  whole triangular solve in one launch (LLT.h:499-505,
//                        PartialPivLU.h:224-271, TriangularSolverMatrix.h)
//   norm kernels         ||A||_1 (PartialPivLU.h:522, LLT.h:434-445)
#pragma once

#include <type_traits>

#include <math.h>

#include "gbs_common.cuh"

namespace gbs {

// --------------------------------------------------------------------- panel LU
// Grid-cooperative: every CTA owns a slice of the panel's rows, each thread
// RPT rows, each row NB values in registers.  One grid barrier per column.
// Scratch layout (global): cand_val[2][P], cand_idx[2][P], cand_row[2][P][NB],
// rowj[2][NB] -- double-buffered by column parity so CTA c can publish column
// j+1's candidate while others still read column j's.
template <typename T, int NB>
struct PanelScratchView {
  T* cand_val;
  int* cand_idx;
  T* cand_row;
  T* rowj;
  __device__ PanelScratchView(void* base, int P)
  {
    char* p = (char*)base;
    cand_val = (T*)p;            p += sizeof(T) * 2 * P;
    cand_row = (T*)p;            p += sizeof(T) * 2 * (size_t)P * NB;
    rowj = (T*)p;                p += sizeof(T) * 2 * NB;
    cand_idx = (int*)p;
  }
};

template <typename T, int NB>
inline size_t panel_scratch_bytes(int P)
{
  return sizeof(T) * (2 * (size_t)P + 2 * (size_t)P * NB + 2 * NB) + sizeof(int) * 2 * (size_t)P + 256;
}

constexpr int kPanelThreads = 256;

template <typename T, int NB, int RPT>
__global__ void __launch_bounds__(kPanelThreads)
panel_lu_kernel(T* __restrict__ a, int64_t lda, int m, int nbc, int k0, int* __restrict__ tr,
                void* scratch, DeviceStatus* st)
{
  const int P = gridDim.x;
  PanelScratchView<T, NB> w(scratch, P);
  const int tid = threadIdx.x;
  const int g = blockIdx.x * kPanelThreads + tid;
  const int G = P * kPanelThreads;
  const int lane = tid & 31, warp = tid >> 5;

  __shared__ T s_u[NB];
  __shared__ T s_oldj[NB];
  __shared__ T s_wval[kPanelThreads / 32];
  __shared__ int s_widx[kPanelThreads / 32];
  __shared__ int s_piv, s_win;

  T v[RPT][NB];
#pragma unroll
  for (int q = 0; q < RPT; ++q) {
    const int r = g + q * G;
#pragma unroll
    for (int c = 0; c < NB; ++c) v[q][c] = (r < m && c < nbc) ? a[(int64_t)c * lda + r] : T(0);
  }

#pragma unroll
  for (int j = 0; j < NB; ++j) {
    if (j >= nbc) break;
    const int par = j & 1;
    // ---- local candidate: first max of |a(r,j)|, r >= j (Visitor.h:173-186)
    T bs = T(-2);
    int bi = 0x7fffffff;
#pragma unroll
    for (int q = 0; q < RPT; ++q) {
      const int r = g + q * G;
      if (r < m && r >= j) {
        T x = v[q][j];
        T s = (r == j) ? ((x != x) ? T(INFINITY) : gbs_abs(x)) : pivot_score(x);
        if (better(s, r, bs, bi)) { bs = s; bi = r; }
      }
    }
    warp_argmax(bs, bi);
    if (lane == 0) { s_wval[warp] = bs; s_widx[warp] = bi; }
    __syncthreads();
    if (warp == 0) {
      bs = lane < kPanelThreads / 32 ? s_wval[lane] : T(-2);
      bi = lane < kPanelThreads / 32 ? s_widx[lane] : 0x7fffffff;
      warp_argmax(bs, bi);
      if (lane == 0) {
        w.cand_val[par * P + blockIdx.x] = bs;
        w.cand_idx[par * P + blockIdx.x] = bi;
        s_win = bi;
      }
    }
    __syncthreads();
    {
      const int winner = s_win;
#pragma unroll
      for (int q = 0; q < RPT; ++q) {
        const int r = g + q * G;
        if (r < m && r == winner) {
#pragma unroll
          for (int c = 0; c < NB; ++c) w.cand_row[((size_t)par * P + blockIdx.x) * NB + c] = v[q][c];
        }
        if (r < m && r == j) {
#pragma unroll
          for (int c = 0; c < NB; ++c) w.rowj[par * NB + c] = v[q][c];
        }
      }
    }
    if (!grid_barrier(st, P)) return;
    // ---- global pivot: every CTA reduces the P candidates itself
    if (warp == 0) {
      T s = T(-2);
      int i = 0x7fffffff, cw = 0;
      for (int c = lane; c < P; c += 32) {
        T sc = ((volatile T*)w.cand_val)[par * P + c];
        int ic = ((volatile int*)w.cand_idx)[par * P + c];
        if (better(sc, ic, s, i)) { s = sc; i = ic; cw = c; }
      }
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        T so = __shfl_xor_sync(0xffffffffu, s, off);
        int io = __shfl_xor_sync(0xffffffffu, i, off);
        int co = __shfl_xor_sync(0xffffffffu, cw, off);
        if (better(so, io, s, i)) { s = so; i = io; cw = co; }
      }
      if (lane == 0) { s_piv = i; s_win = cw; }
    }
    __syncthreads();
    const int p = s_piv;
    for (int c = tid; c < NB; c += kPanelThreads) {
      s_u[c] = ((volatile T*)w.cand_row)[((size_t)par * P + s_win) * NB + c];
      s_oldj[c] = ((volatile T*)w.rowj)[par * NB + c];
    }
    __syncthreads();
    const T piv = s_u[j];
    const bool nz = (piv != T(0));   // biggest_in_corner != 0 (NaN counts as nonzero)
    if (blockIdx.x == 0 && tid == 0) {
      tr[j] = k0 + p;
      if (nz && p != j) st->nb_transpositions += 1;
      if (!nz && st->info < 0) st->info = k0 + j;
    }
#pragma unroll
    for (int q = 0; q < RPT; ++q) {
      const int r = g + q * G;
      if (r >= m) continue;
      if (nz && p != j) {
        if (r == j) {
#pragma unroll
          for (int c = 0; c < NB; ++c) v[q][c] = s_u[c];
        } else if (r == p) {
#pragma unroll
          for (int c = 0; c < NB; ++c) v[q][c] = s_oldj[c];
        }
      }
      if (r > j) {
        if (nz) v[q][j] = v[q][j] / piv;
        const T l = v[q][j];
#pragma unroll
        for (int c = j + 1; c < NB; ++c) v[q][c] = fma(-l, s_u[c], v[q][c]);
      }
    }
    // s_u / s_oldj are rewritten next column only after the next barrier
  }

#pragma unroll
  for (int q = 0; q < RPT; ++q) {
    const int r = g + q * G;
    if (r < m) {
#pragma unroll
      for (int c = 0; c < NB; ++c)
        if (c < nbc) a[(int64_t)c * lda + r] = v[q][c];
    }
  }
}

// --------------------------------------------------------------------- laswp
// Applies the interchanges tr[i0..i1) (absolute row indices, in order, or in
// reverse order when reverse != 0) to the columns [c0, c1) and [c2, c3).
template <typename T>
__global__ void laswp_kernel(T* __restrict__ a, int64_t lda, const int* __restrict__ tr, int i0, int i1,
                             int c0, int c1, int c2, int c3, int reverse)
{
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int n1 = c1 - c0;
  int col;
  if (t < n1) col = c0 + (int)t;
  else if (t < n1 + (c3 - c2)) col = c2 + (int)(t - n1);
  else return;
  T* ac = a + (int64_t)col * lda;
  if (!reverse) {
    for (int i = i0; i < i1; ++i) {
      int p = tr[i];
      if (p != i) { T x = ac[i]; ac[i] = ac[p]; ac[p] = x; }
    }
  } else {
    for (int i = i1 - 1; i >= i0; --i) {
      int p = tr[i];
      if (p != i) { T x = ac[i]; ac[i] = ac[p]; ac[p] = x; }
    }
  }
}

// --------------------------------------------------------------------- TRSM (LU)
// B(nb x ncols) <- L^{-1} B, L unit lower nb x nb (nb <= NB).  One thread per
// column of B, the column in registers, L in shared memory.
template <typename T, int NB>
__global__ void __launch_bounds__(128)
trsm_lunit_kernel(const T* __restrict__ L, int64_t ldl, int nb, T* __restrict__ B, int64_t ldb, int ncols)
{
  __shared__ T sL[NB][NB + 1];
  for (int e = threadIdx.x; e < NB * NB; e += blockDim.x) {
    int i = e % NB, p = e / NB;
    sL[i][p] = (i < nb && p < nb) ? L[(int64_t)p * ldl + i] : T(0);
  }
  __syncthreads();
  int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= ncols) return;
  T* b = B + (int64_t)col * ldb;
  T x[NB];
#pragma unroll
  for (int i = 0; i < NB; ++i) x[i] = i < nb ? b[i] : T(0);
#pragma unroll
  for (int p = 0; p < NB; ++p) {
#pragma unroll
    for (int i = p + 1; i < NB; ++i) x[i] = fma(-sL[i][p], x[p], x[i]);
  }
#pragma unroll
  for (int i = 0; i < NB; ++i)
    if (i < nb) b[i] = x[i];
}

// --------------------------------------------------------------------- GEMM
// C(M x N) -= op(A)(M x K) * op(B)(K x N) with op given by element strides:
// A(i,k) = A[i*a_rs + k*a_cs], B(k,j) = B[k*b_rs + j*b_cs].  lower != 0 keeps
// only the lower triangle of C (i >= j; SYRK).  Skips all work when
// `stop_flag` is non-null and >= 0 (an earlier LLT block failed).
template <typename T, int BM, int BN, int BK, int TM, int TN>
__global__ void __launch_bounds__((BM / TM) * (BN / TN))
gemm_sub_kernel(int M, int N, int K, const T* __restrict__ A, int64_t a_rs, int64_t a_cs,
                const T* __restrict__ B, int64_t b_rs, int64_t b_cs, T* __restrict__ C, int64_t ldc,
                int lower, const int* stop_flag)
{
  griddep_launch_dependents();
  griddep_wait();
  constexpr int TX = BN / TN, TY = BM / TM, NT = TX * TY;
  const int bm = blockIdx.y * BM, bn = blockIdx.x * BN;
  if (lower && bn >= bm + BM) return;                 // tile strictly above the diagonal
  if (stop_flag && ld_volatile_i32(stop_flag) >= 0) return;
  __shared__ T As[BK][BM + 1];
  __shared__ T Bs[BK][BN + 1];
  const int tid = threadIdx.x;
  const int tx = tid % TX, ty = tid / TX;
  T acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) acc[i][j] = T(0);

  for (int k0 = 0; k0 < K; k0 += BK) {
    for (int e = tid; e < BM * BK; e += NT) {
      int i = e % BM, kk = e / BM;
      int gi = bm + i, gk = k0 + kk;
      As[kk][i] = (gi < M && gk < K) ? A[(int64_t)gi * a_rs + (int64_t)gk * a_cs] : T(0);
    }
    for (int e = tid; e < BN * BK; e += NT) {
      int kk = e % BK, j = e / BK;
      int gj = bn + j, gk = k0 + kk;
      Bs[kk][j] = (gj < N && gk < K) ? B[(int64_t)gk * b_rs + (int64_t)gj * b_cs] : T(0);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      T af[TM], bf[TN];
#pragma unroll
      for (int i = 0; i < TM; ++i) af[i] = As[kk][ty + i * TY];
#pragma unroll
      for (int j = 0; j < TN; ++j) bf[j] = Bs[kk][tx + j * TX];
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = fma(af[i], bf[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int j = 0; j < TN; ++j) {
    int gj = bn + tx + j * TX;
    if (gj >= N) continue;
#pragma unroll
    for (int i = 0; i < TM; ++i) {
      int gi = bm + ty + i * TY;
      if (gi >= M) continue;
      if (lower && gi < gj) continue;
      T* c = C + (int64_t)gj * ldc + gi;
      *c = *c - acc[i][j];
    }
  }
}

// --------------------------------------------------------------------- LLT diag
// Cholesky of the bs x bs diagonal block in shared memory, the reference's
// unblocked algorithm (LLT.h:305-328: x = a_kk - ||l_k||^2, fail if x <= 0,
// x = sqrt(x), column divided by x) in right-looking order with a one-column
// look-ahead: while six warps apply column k to the trailing columns k+2..,
// warp 0 applies it to column k+1 alone, then checks, square-roots and scales
// column k+1, so one barrier per column separates the steps and the square
// root overlaps the bulk of the update.  The bulk is dealt out evenly: the
// trailing triangle is a suffix of the packed column-major order, and a
// table gives each packed element's (row, column), so every FP64 warp
// instruction (64 cycles on GB300 whatever the active lanes) carries 32
// elements.  Every element sees the same FMAs in the same order as in a
// plain right-looking sweep.  In FP64 the column is
// scaled by the reciprocal square root (within an ulp of the reference's
// division, one long-latency sequence instead of two); FP32 divides by the
// square root as the reference does.  On failure writes k0 + k into st->info
// and writes back only the columns already final (the trailing columns in
// global memory were never touched, as the reference's early return leaves
// them).  Only the lower triangle is read or written.
// Dynamic smem: potrf_diag_smem<T>(bs) (the block and the element table);
// 256 threads, bs <= 128.
template <typename T>
__host__ __device__ constexpr size_t potrf_diag_smem(int bs)
{
  return sizeof(T) * (size_t)bs * (bs + 1) + sizeof(unsigned short) * (size_t)(bs * (bs + 1) / 2);
}

// Column k's own step (warp 0): check, then scale.  FP64 keeps x_kk in sd[k]
// and takes the diagonal's square roots at the end, all at once (a 730-cycle
// sqrt per column would sit on warp 0's chain); FP32 writes sqrt(x_kk).
template <typename T>
__device__ __forceinline__ bool llt_diag_column(T* s, T* sd, int ld, int bs, int k, int lane)
{
  const T d = s[k * ld + k];
  if (!(d > T(0)) && !(d != d)) return false;         // x <= 0 (a NaN does not fail, as in the reference)
  if constexpr (std::is_same<T, double>::value) {
    const T r = rsqrt(d);
    for (int i = k + 1 + lane; i < bs; i += 32) s[k * ld + i] *= r;
    if (lane == 0) sd[k] = d;
  } else {
    const T x = sqrt(d);
    for (int i = k + 1 + lane; i < bs; i += 32) s[k * ld + i] = s[k * ld + i] / x;
    if (lane == 0) s[k * ld + k] = x;
  }
  return true;
}

template <typename T>
__global__ void __launch_bounds__(256)
potrf_diag_kernel(T* __restrict__ a, int64_t lda, int bs, int k0, DeviceStatus* st)
{
  griddep_launch_dependents();
  griddep_wait();
  if (st->info >= 0) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* s = (T*)smem_raw;
  const int ld = bs + 1;
  const int tid = threadIdx.x, nt = blockDim.x, warp = tid >> 5, lane = tid & 31;
  __shared__ int s_fail;
  __shared__ T sd[128];                                 // FP64: x_kk, square-rooted at the end
  // tab[e] = (i << 8) | j for the e-th element (i >= j) of the packed
  // column-major lower triangle: the trailing triangle of step k (j >= k+2)
  // is the suffix from pstart(k+2), so the update deals it out evenly
  const int tot = bs * (bs + 1) / 2;
  unsigned short* tab = (unsigned short*)(s + bs * ld);
  auto pstart = [bs](int j) { return j * bs - j * (j - 1) / 2; };
  for (int e = tid; e < bs * bs; e += nt) {
    const int i = e % bs, j = e / bs;
    if (i >= j) s[j * ld + i] = a[(int64_t)j * lda + i];
  }
  for (int j = warp; j < bs; j += nt / 32)
    for (int i = j + lane; i < bs; i += 32) tab[pstart(j) + i - j] = (unsigned short)((i << 8) | j);
  if (tid == 0) s_fail = -1;
  __syncthreads();
  if (warp == 0 && !llt_diag_column(s, sd, ld, bs, 0, lane) && lane == 0) s_fail = 0;
  __syncthreads();
  // the trailing update runs on warps 1-3 and 5-7: warp 4 would share warp 0's
  // FP64 unit (sub-partition 0) and slow its chain
  const int bw = warp < 4 ? warp - 1 : warp - 2;        // 0..5 for warps 1-3, 5-7
  const int t = bw * 32 + lane, nw = 192;
  auto finish_diag = [&](int upto) {                    // FP64: l_kk = sqrt(x_kk) for k < upto
    if constexpr (std::is_same<T, double>::value) {
      __syncthreads();
      for (int k = tid; k < upto; k += nt) s[k * ld + k] = sqrt(sd[k]);
      __syncthreads();
    }
  };
  for (int k = 0; k < bs; ++k) {
    const int f = s_fail;
    if (f >= 0) {                                       // column f failed; columns < f are final
      finish_diag(f);
      if (tid == 0) st->info = k0 + f;
      for (int e = tid; e < bs * f; e += nt) {
        const int i = e % bs, j = e / bs;
        if (i >= j) a[(int64_t)j * lda + i] = s[j * ld + i];
      }
      return;
    }
    if (k + 1 >= bs) break;
    if (warp == 0) {
      // column k+1: a_{i,k+1} -= l_ik l_{k+1,k}, then its own step
      const T lj = s[k * ld + k + 1];
      for (int i = k + 1 + lane; i < bs; i += 32) s[(k + 1) * ld + i] = fma(-s[k * ld + i], lj, s[(k + 1) * ld + i]);
      __syncwarp();
      if (!llt_diag_column(s, sd, ld, bs, k + 1, lane) && lane == 0) s_fail = k + 1;
    } else if (warp != 4) {
      // columns k+2..: a_ij -= l_ik l_jk for k+2 <= j <= i, two elements per thread at a time
      int e = pstart(k + 2) + t;
      for (; e + nw < tot; e += 2 * nw) {
        const unsigned v0 = tab[e], v1 = tab[e + nw];
        const int i0 = v0 >> 8, j0 = v0 & 255, i1 = v1 >> 8, j1 = v1 & 255;
        const T a0 = s[j0 * ld + i0], a1 = s[j1 * ld + i1];
        const T p0 = s[k * ld + i0], q0 = s[k * ld + j0], p1 = s[k * ld + i1], q1 = s[k * ld + j1];
        s[j0 * ld + i0] = fma(-p0, q0, a0);
        s[j1 * ld + i1] = fma(-p1, q1, a1);
      }
      if (e < tot) {
        const unsigned v0 = tab[e];
        const int i0 = v0 >> 8, j0 = v0 & 255;
        s[j0 * ld + i0] = fma(-s[k * ld + i0], s[k * ld + j0], s[j0 * ld + i0]);
      }
    }
    __syncthreads();
  }
  finish_diag(bs);
  for (int e = tid; e < bs * bs; e += nt) {
    const int i = e % bs, j = e / bs;
    if (i >= j) a[(int64_t)j * lda + i] = s[j * ld + i];
  }
}

// --------------------------------------------------------------------- LLT TRSM
// X(m x bs) <- X L^{-T}, L lower bs x bs.  One thread per row of X; the CTA's
// rows and L live in shared memory; in FP64 the reciprocals of L's diagonal
// are taken once per CTA, so a column step is a dot product and a multiply
// (FP32 divides, as the reference does).
// Dynamic smem: (bs*(bs+1) + bs*RT + bs)*sizeof(T).
template <typename T, int RT>
__global__ void __launch_bounds__(RT)
trsm_rlt_kernel(const T* __restrict__ L, int64_t ldl, int bs, T* __restrict__ X, int64_t ldx, int m,
                const DeviceStatus* st)
{
  if (st && ld_volatile_i32(&st->info) >= 0) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* sL = (T*)smem_raw;              // sL[j*(bs+1) + l] = L(j,l)
  T* sX = sL + bs * (bs + 1);        // sX[c*RT + t]
  T* sR = sX + bs * RT;              // sR[j] = 1 / L(j,j)
  const int ldL = bs + 1;
  for (int e = threadIdx.x; e < bs * bs; e += RT) {
    int j = e % bs, l = e / bs;
    if (j >= l) sL[j * ldL + l] = L[(int64_t)l * ldl + j];
  }
  for (int j = threadIdx.x; j < bs; j += RT) sR[j] = std::is_same<T, double>::value ? T(1) / L[(int64_t)j * ldl + j] : L[(int64_t)j * ldl + j];
  const int r0 = blockIdx.x * RT;
  for (int e = threadIdx.x; e < bs * RT; e += RT) {
    int t = e % RT, c = e / RT;
    int r = r0 + t;
    sX[c * RT + t] = r < m ? X[(int64_t)c * ldx + r] : T(0);
  }
  __syncthreads();
  const int t = threadIdx.x;
  for (int j = 0; j < bs; ++j) {
    T s0 = sX[j * RT + t], s1 = T(0), s2 = T(0), s3 = T(0);   // four chains: FMA latency, not issue, bounds this
    int l = 0;
    for (; l + 3 < j; l += 4) {
      s0 = fma(-sX[l * RT + t], sL[j * ldL + l], s0);
      s1 = fma(-sX[(l + 1) * RT + t], sL[j * ldL + l + 1], s1);
      s2 = fma(-sX[(l + 2) * RT + t], sL[j * ldL + l + 2], s2);
      s3 = fma(-sX[(l + 3) * RT + t], sL[j * ldL + l + 3], s3);
    }
    for (; l < j; ++l) s0 = fma(-sX[l * RT + t], sL[j * ldL + l], s0);
    const T sj = (s0 + s1) + (s2 + s3);
    if constexpr (std::is_same<T, double>::value) sX[j * RT + t] = sj * sR[j];   // FP64: no division on the chain
    else sX[j * RT + t] = sj / sR[j];
  }
  __syncthreads();
  for (int e = threadIdx.x; e < bs * RT; e += RT) {
    int tt = e % RT, c = e / RT;
    int r = r0 + tt;
    if (r < m) X[(int64_t)c * ldx + r] = sX[c * RT + tt];
  }
}

// X(m x bs) <- X L^{-T} in 16-column blocks, for latency: per block, every
// (row, column) pair first subtracts the finished columns' contribution (a
// dot product, all pairs in parallel), then the block is finished
// right-looking with its 16 columns spread over the 8 warps (a multiply, a
// barrier and one FMA per step on the dependent chain).  RT <= 32 rows per
// CTA, 256 threads, bs <= 128, the last block may be narrower.  FP64 multiplies by the reciprocals of L's
// diagonal, FP32 divides.  Dynamic smem: (bs*(bs+1) + bs*RT + bs)*sizeof(T).
template <typename T, int RT>
__global__ void __launch_bounds__(256)
trsm_rlt_blocked_kernel(const T* __restrict__ L, int64_t ldl, int bs, T* __restrict__ X, int64_t ldx, int m,
                        const DeviceStatus* st)
{
  griddep_launch_dependents();
  griddep_wait();
  constexpr int W = 16;
  constexpr bool kRecip = std::is_same<T, double>::value;
  if (st && ld_volatile_i32(&st->info) >= 0) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* sL = (T*)smem_raw;              // sL[j*(bs+1) + l] = L(j,l)
  T* sX = sL + bs * (bs + 1);        // sX[c*RT + t]
  T* sR = sX + bs * RT;              // FP64: 1 / L(j,j); FP32: L(j,j)
  const int ldL = bs + 1, tid = threadIdx.x, nt = blockDim.x;
  for (int e = tid; e < bs * bs; e += nt) {
    const int j = e % bs, l = e / bs;
    if (j >= l) sL[j * ldL + l] = L[(int64_t)l * ldl + j];
  }
  for (int j = tid; j < bs; j += nt) sR[j] = kRecip ? T(1) / L[(int64_t)j * ldl + j] : L[(int64_t)j * ldl + j];
  const int r0 = blockIdx.x * RT;
  for (int e = tid; e < bs * RT; e += nt) {
    const int t = e % RT, c = e / RT;
    const int r = r0 + t;
    sX[c * RT + t] = r < m ? X[(int64_t)c * ldx + r] : T(0);
  }
  __syncthreads();
  for (int jb = 0; jb < bs; jb += W) {
    const int wb = min(W, bs - jb);
    if (jb > 0) {
      for (int e = tid; e < RT * wb; e += nt) {       // x_rc -= sum_{l < jb} x_rl L(c,l)
        const int t = e % RT, c = jb + e / RT;
        T s0 = sX[c * RT + t], s1 = T(0), s2 = T(0), s3 = T(0);
        for (int l = 0; l < jb; l += 4) {
          s0 = fma(-sX[l * RT + t], sL[c * ldL + l], s0);
          s1 = fma(-sX[(l + 1) * RT + t], sL[c * ldL + l + 1], s1);
          s2 = fma(-sX[(l + 2) * RT + t], sL[c * ldL + l + 2], s2);
          s3 = fma(-sX[(l + 3) * RT + t], sL[c * ldL + l + 3], s3);
        }
        sX[c * RT + t] = (s0 + s1) + (s2 + s3);
      }
      __syncthreads();
    }
    // the block's own columns, right-looking: warp w owns columns jb+w and
    // jb+w+8 (lane = row); a step is the owner's multiply, a barrier, and
    // one FMA per later column, so no warp issues the block's FMAs alone
    {
      const int w = tid >> 5, ln = tid & 31;
      const int ca = w, cb = w + 8;                    // owned columns within the block
      T xa = T(0), xb = T(0);
      if (ln < RT) {
        if (ca < wb) xa = sX[(jb + ca) * RT + ln];
        if (cb < wb) xb = sX[(jb + cb) * RT + ln];
      }
      for (int c = 0; c < wb; ++c) {
        if (ln < RT && (c == ca || c == cb)) {         // the owner finishes column c
          T& xc = c == ca ? xa : xb;
          xc = kRecip ? xc * sR[jb + c] : xc / sR[jb + c];
          sX[(jb + c) * RT + ln] = xc;
        }
        __syncthreads();
        if (ln < RT) {
          const T xc = sX[(jb + c) * RT + ln];
          if (ca > c && ca < wb) xa = fma(-xc, sL[(jb + ca) * ldL + jb + c], xa);
          if (cb > c && cb < wb) xb = fma(-xc, sL[(jb + cb) * ldL + jb + c], xb);
        }
      }
    }
    __syncthreads();
  }
  for (int e = tid; e < bs * RT; e += nt) {
    const int t = e % RT, c = e / RT;
    const int r = r0 + t;
    if (r < m) X[(int64_t)c * ldx + r] = sX[c * RT + t];
  }
}

// --------------------------------------------------------------------- persistent TRSM
// op(Tri) X = B for up to RC right-hand sides in ONE launch.  Block rows of NB
// are handed out in solve order by a ticket counter.  Block i subtracts
// op(Tri)(i,j) x_j for every earlier block j: it waits (bounded) for the first
// block it still needs, takes every further block already finished (up to
// SUPER of them) and applies them as one streamed super-tile (all loads of the
// tile issued before the barrier), so a block that fell behind catches up in a
// few passes.  It then solves its diagonal block with one warp per right-hand
// side (rows spread over lanes, shuffles carry x_r), writes x_i and raises its
// flag.  A CTA only takes a ticket while running and only waits on lower
// tickets, so the lowest unfinished block always progresses.  work: [0] ticket
// counter, [1] unused, [2..] one ready flag per block; zeroed before launch.
// err: timeout flag, set to 1 when a wait runs past limit_ns and left set
// across launches until the host reads it.  Dynamic shared memory:
// trsm_persistent_smem<T, NB, RC>().
template <typename T, int NB>
struct TrsmSuper { static constexpr int value = 256 / NB; };

template <typename T, int NB, int RC>
constexpr size_t trsm_persistent_smem()
{
  constexpr int K = TrsmSuper<T, NB>::value * NB;
  return sizeof(T) * ((size_t)K * (NB + 1) + (size_t)K * RC + (size_t)NB * RC + (size_t)NB * (NB + 1));
}

// dinv (may be null): the inverses of the diagonal blocks of op(Tri), block b
// at dinv + b NB^2, NB x NB column-major (zero beyond the block's rows and
// columns); with them a block's own step is X_b = Dinv_b Y_b, a product with
// independent FMAs instead of an NB-step substitution.
template <typename T, int NB, int RC>
__global__ void __launch_bounds__(RC * 32, 2)
trsm_persistent_kernel(int n, int nrhs, const T* __restrict__ tri, int64_t rs, int64_t cs, int forward, int unit,
                       T* B, int64_t ldb, int* work, const T* __restrict__ dinv, int* err, uint64_t limit_ns)
{
  constexpr int PER = NB / 32;
  constexpr int SUPER = TrsmSuper<T, NB>::value;
  constexpr int KMAX = SUPER * NB;
  constexpr int G = (RC * 32) / NB;          // right-hand-side groups of the accumulation
  constexpr int CPT = RC / G;                // right-hand sides per thread
  static_assert(G * NB == RC * 32 && CPT * G == RC, "thread mapping");
  const int nblk = (n + NB - 1) / NB;
  int* counter = work;
  int* flags = work + 2;
  const uint64_t limit = effective_limit(limit_ns);
  extern __shared__ __align__(16) unsigned char trsm_sm[];
  T(*sT)[NB + 1] = reinterpret_cast<T(*)[NB + 1]>(trsm_sm);                         // [KMAX][NB+1], k-major
  T(*sX)[RC] = reinterpret_cast<T(*)[RC]>(trsm_sm + sizeof(T) * KMAX * (NB + 1));     // [KMAX][RC]
  T(*sY)[RC] = reinterpret_cast<T(*)[RC]>(trsm_sm + sizeof(T) * (KMAX * (NB + 1) + KMAX * RC));
  T(*sD)[NB + 1] = reinterpret_cast<T(*)[NB + 1]>(trsm_sm + sizeof(T) * (KMAX * (NB + 1) + KMAX * RC + NB * RC));
  __shared__ int s_t, s_ok, s_hi;
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int warp = tid >> 5, lane = tid & 31;
  const int ar = tid % NB, ag = tid / NB;     // accumulation: row, right-hand-side group
  const bool unit_rows_fast = (rs == 1);
  for (;;) {
    if (tid == 0) s_t = atomicAdd(counter, 1);
    __syncthreads();
    const int t = s_t;
    if (t >= nblk) break;
    const int bi = forward ? t : nblk - 1 - t;
    const int i0 = bi * NB, ni = min(NB, n - i0);
    // the diagonal tile (or its inverse) and the first off-diagonal tile do
    // not depend on any other block: load them before waiting
    if (dinv) {
      const T* db = dinv + (int64_t)bi * NB * NB;
      for (int e = tid; e < NB * NB; e += nthr) sD[e % NB][e / NB] = db[e];
    } else {
      for (int e = tid; e < NB * NB; e += nthr) {
        int r, c;
        if (unit_rows_fast) { r = e % NB; c = e / NB; } else { c = e % NB; r = e / NB; }
        sD[r][c] = (r < ni && c < ni) ? tri[(int64_t)(i0 + r) * rs + (int64_t)(i0 + c) * cs] : T(0);
      }
    }
    T acc[CPT];
#pragma unroll
    for (int q = 0; q < CPT; ++q) {
      const int c = ag + q * G;
      acc[q] = (ar < ni && c < nrhs) ? B[(int64_t)c * ldb + i0 + ar] : T(0);
    }
    int done = 0;
    int loaded = 0;                            // T tiles of blocks done..loaded-1 already in sT
    auto load_tiles = [&](int from, int to) {  // op(Tri) columns of blocks [from, to) into sT rows (b - done) * NB
      const int K = (to - from) * NB, base = (from - done) * NB;
#pragma unroll 8
      for (int e = tid; e < NB * K; e += nthr) {
        int r, kk;
        if (unit_rows_fast) { r = e % NB; kk = e / NB; } else { kk = e % K; r = e / K; }
        const int jb = from + kk / NB, w = kk % NB;
        const int bj = forward ? jb : nblk - 1 - jb;
        const int col = bj * NB + w;
        sT[base + kk][r] = (r < ni && col < n) ? tri[(int64_t)(i0 + r) * rs + (int64_t)col * cs] : T(0);
      }
    };
    while (done < t) {
      if (loaded == done) {                    // prefetch the tile the wait below is for
        load_tiles(done, done + 1);
        loaded = done + 1;
      }
      if (tid == 0) {
        int ok = 1;
        const int bj0 = forward ? done : nblk - 1 - done;
        if (ld_acquire_u32((const unsigned int*)&flags[bj0]) == 0u) {
          const uint64_t t0 = globaltimer_ns();
          unsigned int spins = 0;
          while (ld_acquire_u32((const unsigned int*)&flags[bj0]) == 0u) {
            if ((++spins & 63u) == 0 &&
                (ld_volatile_i32(err) || globaltimer_ns() - t0 > limit)) {
              atomicExch(err, 1);
              ok = 0;
              break;
            }
            __nanosleep(32);
          }
        }
        int hi = done + 1;
        while (ok && hi < t && hi - done < SUPER &&
               ld_acquire_u32((const unsigned int*)&flags[forward ? hi : nblk - 1 - hi]) != 0u)
          ++hi;
        s_ok = ok;
        s_hi = hi;
      }
      __syncthreads();
      if (!s_ok) return;
      const int hi = s_hi;
      const int K = (hi - done) * NB;
      if (hi > loaded) load_tiles(loaded, hi);
#pragma unroll 4
      for (int e = tid; e < K * RC; e += nthr) {
        const int kk = e % K, c = e / K;
        const int jb = done + kk / NB, w = kk % NB;
        const int bj = forward ? jb : nblk - 1 - jb;
        const int col = bj * NB + w;
        sX[kk][c] = (col < n && c < nrhs) ? __ldcg(&B[(int64_t)c * ldb + col]) : T(0);
      }
      __syncthreads();
      for (int k0 = 0; k0 < K && ag < nrhs; k0 += NB) {   // one partial sum per tile: rounding grows with NB, not with n
        // (groups beyond nrhs skip: an FP64 instruction costs its unit 64 cycles even on zero columns)
        T part[CPT];
#pragma unroll
        for (int q = 0; q < CPT; ++q) part[q] = T(0);
#pragma unroll 8
        for (int kk = k0; kk < k0 + NB; ++kk) {
          const T tv = sT[kk][ar];
#pragma unroll
          for (int q = 0; q < CPT; ++q) part[q] = fma(tv, sX[kk][ag + q * G], part[q]);
        }
#pragma unroll
        for (int q = 0; q < CPT; ++q) acc[q] -= part[q];
      }
      __syncthreads();
      done = hi;
      loaded = hi;
    }
#pragma unroll
    for (int q = 0; q < CPT; ++q) sY[ar][ag + q * G] = acc[q];
    if (dinv) {                                // X_b = Dinv_b Y_b
      __syncthreads();
      T out[CPT];
#pragma unroll
      for (int q = 0; q < CPT; ++q) out[q] = T(0);
#pragma unroll 8
      for (int k = 0; k < NB && ag < nrhs; ++k) {
        const T dv = sD[ar][k];
#pragma unroll
        for (int q = 0; q < CPT; ++q) out[q] = fma(dv, sY[k][ag + q * G], out[q]);
      }
#pragma unroll
      for (int q = 0; q < CPT; ++q) {
        const int c = ag + q * G;
        if (ar < ni && c < nrhs) B[(int64_t)c * ldb + i0 + ar] = out[q];
      }
      __syncthreads();
      if (tid == 0) st_release_u32((unsigned int*)&flags[bi], 1u);
      continue;
    }
    __syncthreads();
    if (warp < nrhs) {
      // FP64: reciprocals of the diagonal, taken off the substitution's chain
      // (within an ulp of the division); FP32 divides
      constexpr bool kRecip = std::is_same<T, double>::value;
      T yl[PER], rd[PER];
#pragma unroll
      for (int p = 0; p < PER; ++p) {
        yl[p] = sY[lane + 32 * p][warp];
        rd[p] = (unit || lane + 32 * p >= ni) ? T(1) : kRecip ? T(1) / sD[lane + 32 * p][lane + 32 * p]
                                                                : sD[lane + 32 * p][lane + 32 * p];
      }
      if (forward) {
#pragma unroll
        for (int r = 0; r < NB; ++r) {
          if (r < ni) {
            const T yr = __shfl_sync(0xffffffffu, yl[r / 32], r % 32), dr = __shfl_sync(0xffffffffu, rd[r / 32], r % 32);
            const T xr = kRecip ? yr * dr : yr / dr;
#pragma unroll
            for (int p = 0; p < PER; ++p) {
              const int row = lane + 32 * p;
              if (row > r && row < ni) yl[p] = fma(-sD[row][r], xr, yl[p]);
            }
            if (lane == r % 32) yl[r / 32] = xr;
          }
        }
      } else {
#pragma unroll
        for (int r = NB - 1; r >= 0; --r) {
          if (r < ni) {
            const T yr = __shfl_sync(0xffffffffu, yl[r / 32], r % 32), dr = __shfl_sync(0xffffffffu, rd[r / 32], r % 32);
            const T xr = kRecip ? yr * dr : yr / dr;
#pragma unroll
            for (int p = 0; p < PER; ++p) {
              const int row = lane + 32 * p;
              if (row < r) yl[p] = fma(-sD[row][r], xr, yl[p]);
            }
            if (lane == r % 32) yl[r / 32] = xr;
          }
        }
      }
#pragma unroll
      for (int p = 0; p < PER; ++p) sY[lane + 32 * p][warp] = yl[p];
    }
    __syncthreads();
    for (int e = tid; e < NB * RC; e += nthr) {
      const int r = e % NB, c = e / NB;
      if (r < ni && c < nrhs) B[(int64_t)c * ldb + i0 + r] = sY[r][c];
    }
    __syncthreads();
    if (tid == 0) st_release_u32((unsigned int*)&flags[bi], 1u);
  }
}


// --------------------------------------------------------------------- norms
__device__ __forceinline__ void atomic_max_nonneg(double* addr, double v)
{
  if (!(v >= 0.0)) return;
  atomicMax((unsigned long long*)addr, (unsigned long long)__double_as_longlong(v));
}

// max_j sum_i |a(i,j)| (one warp per column); out must start at 0.
template <typename T>
__global__ void l1_norm_kernel(const T* __restrict__ a, int64_t lda, int m, int n, double* out)
{
  int col = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  int lane = threadIdx.x & 31;
  if (col >= n) return;
  const T* c = a + (int64_t)col * lda;
  T s = T(0);
  for (int i = lane; i < m; i += 32) s += gbs_abs(c[i]);
  s = warp_sum(s);
  if (lane == 0) atomic_max_nonneg(out, (double)s);
}

// Symmetric ||A||_1 reading only the stored triangle (LLT.h:434-445).
template <typename T>
__global__ void sym_l1_norm_kernel(const T* __restrict__ a, int64_t lda, int n, int upper, double* out)
{
  int col = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  int lane = threadIdx.x & 31;
  if (col >= n) return;
  T s = T(0);
  if (!upper) {
    for (int i = col + lane; i < n; i += 32) s += gbs_abs(a[(int64_t)col * lda + i]);
    for (int j = lane; j < col; j += 32) s += gbs_abs(a[(int64_t)j * lda + col]);
  } else {
    for (int i = lane; i < col; i += 32) s += gbs_abs(a[(int64_t)col * lda + i]);
    for (int j = col + lane; j < n; j += 32) s += gbs_abs(a[(int64_t)j * lda + col]);
  }
  s = warp_sum(s);
  if (lane == 0) atomic_max_nonneg(out, (double)s);
}

// Copies an m x n column-major block (lda -> ldb), optionally converting type.
template <typename TI, typename TO>
__global__ void copy_matrix_kernel(const TI* __restrict__ a, int64_t lda, TO* __restrict__ b, int64_t ldb,
                                   int m, int n)
{
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t total = (int64_t)m * n;
  for (; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    int i = (int)(t % m), j = (int)(t / m);
    b[(int64_t)j * ldb + i] = (TO)a[(int64_t)j * lda + i];
  }
}

// out(j,i) = in(i,j) for i,j in the stored triangle: moves the upper triangle
// of `a` to the lower triangle of `b` (to_lower) or back.
template <typename T>
__global__ void transpose_triangle_kernel(const T* __restrict__ a, int64_t lda, T* __restrict__ b, int64_t ldb,
                                          int n, int to_lower)
{
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t total = (int64_t)n * n;
  for (; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    int i = (int)(t % n), j = (int)(t / n);
    if (to_lower) { if (i >= j) b[(int64_t)j * ldb + i] = a[(int64_t)i * lda + j]; }
    else          { if (i <= j) b[(int64_t)j * ldb + i] = a[(int64_t)i * lda + j]; }
  }
}

}  // namespace gbs
