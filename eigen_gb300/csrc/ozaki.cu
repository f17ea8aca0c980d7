// FP64-accurate residual R = B - A X on the bf16 tensor cores (Ozaki scheme).
//
// Ozaki, Ogita, Oishi, Rump, "Error-free transformations of matrix
// multiplication by using fast routines of matrix multiplication and its
// applications", Numer. Algorithms 59 (2012); Mukunoki, Ozaki, Ogita, Imamura,
// "DGEMM using Tensor Cores, and Its Accurate and Reproducible Versions",
// ISC 2020.  Here:
//   * every row r of A is scaled by 2^-e_r (max_k |A(r,k)| < 2^e_r) and cut
//     into 8 digit slices A_i of 7 bits: A(r,k) = 2^e_r sum_i d_i(r,k) 2^-7(i+1)
//     with integer digits |d_i| <= 127 (truncation toward zero, exact in FP64);
//     every column c of X likewise with 2^f_c.  Both are exact in bf16.
//   * P_ij = A_i X_j is an integer matrix; over a K-chunk of 1024 every partial
//     sum is below 1024 * 127^2 < 2^24, so the tensor core's FP32 accumulation
//     is exact.  The chunk sums are added as int32, folded per slice pair into
//     FP64 as (A X)(r,c) = 2^(e_r + f_c - 14) sum_ij P_ij(r,c) 2^-7(i+j).
//   * The only rounding is the digit tail beyond 56 bits (elements more than
//     three binades below their row or column maximum) and the final FP64
//     additions: the result is as accurate as an FP64 GEMV (n u |A||X|).
// One MMA computes A_i against all 8 X slices at once: the B operand stacks
// X_j for the 16 right-hand sides as N = 8 x 16 = 128 rows.
//
// Kernel layout (one CTA per (128-row block, K range)):
//   warp 0      TMA producer: one 128-byte K-slice of A_i (128 rows) and of the
//               stacked X slices (128 rows) per stage, 128B-swizzled, 6 stages
//   warp 1      TMEM allocator + MMA issuer: 4 x tcgen05.mma kind::f16 (bf16,
//               M=128, N=128) per stage; one accumulator per (slice i, chunk),
//               double-buffered in TMEM
//   warps 2-5   epilogue: tcgen05.ld of each accumulator, int32 accumulation
//               over the chunks, FP64 fold per slice, partial R written per K range
// Every wait is bounded; on expiry the kernel sets the timeout flag, drains its
// copies, frees TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>

#include "dense_driver.cuh"
#include "gbs_profile.cuh"
#include "ozaki.cuh"
#include "tc_ptx.cuh"

namespace gbs {
namespace {

constexpr int OZ_BM = 128;                 // rows of A per tile
constexpr int OZ_RHS = 16;                 // right-hand sides per product
constexpr int OZ_SLICES = 8;               // digit slices of A and of X
constexpr int OZ_BN = OZ_SLICES * OZ_RHS;  // stacked X slices: 128 MMA columns
constexpr int OZ_DIGIT = 7;                // bits per digit
constexpr int OZ_CHUNK = 1024;             // K of one exact FP32 accumulation
constexpr int OZ_ATOM = 128;               // bytes of K per stage (one swizzle atom)
constexpr int OZ_KS = OZ_ATOM / 2;         // bf16 elements of K per stage
constexpr int OZ_STAGES = 6;
constexpr int OZ_THREADS = 192;
constexpr int OZ_A_STAGE = OZ_BM * OZ_ATOM;
constexpr int OZ_B_STAGE = OZ_BN * OZ_ATOM;
constexpr int OZ_STAGE_BYTES = OZ_A_STAGE + OZ_B_STAGE;
constexpr int OZ_SMEM = OZ_STAGES * OZ_STAGE_BYTES + 1024 + 256;
constexpr uint32_t OZ_TMEM_COLS = 2 * OZ_BN;
constexpr int OZ_MAX_CHUNKS_PER_CTA = 64;  // int32 sums of up to 64 chunks: < 2^30
static_assert((int64_t)OZ_CHUNK * 127 * 127 < (1 << 24), "chunk sums must stay exact in FP32");

constexpr unsigned long long kNonFiniteBits = 0x7FF0000000000000ull;

// Exponent e with |v| < 2^e for the largest magnitude v (0 when v = 0): the
// biased exponent field plus one for a normal number, and for a subnormal
// the position of its highest set mantissa bit.
__device__ __forceinline__ int bound_exponent(unsigned long long maxbits)
{
  if (maxbits == 0) return 0;
  const int ef = (int)(maxbits >> 52);
  if (ef > 0) return ef - 1022;                          // 1.f x 2^(ef - 1023) < 2^(ef - 1022)
  return (63 - __clzll(maxbits)) - 1073;                 // highest mantissa bit b: v < 2^(b + 1 - 1074)
}

// The 56-bit fixed-point magnitude F = trunc(|v| 2^(56 - e)) of a finite v
// with |v| < 2^e, from v's bits (integer shifts only), and its sign.
__device__ __forceinline__ unsigned long long fixed56(double v, int e, bool* neg)
{
  const unsigned long long bits = (unsigned long long)__double_as_longlong(v);
  *neg = (bits >> 63) != 0;
  const int ef = (int)((bits >> 52) & 0x7FF);
  const unsigned long long frac = bits & 0xFFFFFFFFFFFFFull;
  if (ef == 0 && frac == 0) return 0;
  const unsigned long long m = ef ? (frac | (1ull << 52)) : frac;   // |v| = m 2^(E), E = max(ef, 1) - 1075
  const int shift = (ef ? ef : 1) - 1075 - e + 56;                  // F = m 2^shift < 2^56: shift <= 55
  if (shift >= 0) return m << shift;
  return shift <= -64 ? 0ull : (m >> (-shift));
}

// Digit i (most significant first) of F: F = sum_i d_i 2^(7 (7 - i)).
__device__ __forceinline__ __nv_bfloat16 digit_bf16(unsigned long long F, bool neg, int i)
{
  const int d = (int)((F >> (OZ_DIGIT * (OZ_SLICES - 1 - i))) & ((1u << OZ_DIGIT) - 1));
  return __float2bfloat16_rn((float)(neg ? -d : d));    // |d| <= 127: exact
}

// Row maxima of |A| as bit patterns (for non-negative doubles the bit order is
// the value order; NaN and infinities compare above every finite value).  One
// thread per row over a range of columns (coalesced down the columns), one
// atomic per thread.
__global__ void oz_row_absmax_kernel(int n, const double* __restrict__ A, int64_t lda, int kspan,
                                     unsigned long long* __restrict__ rowmax)
{
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const int k0 = blockIdx.y * kspan, k1 = min(n, k0 + kspan);
  unsigned long long m = 0;
  for (int k = k0; k < k1; ++k)
    m = max(m, (unsigned long long)__double_as_longlong(A[(int64_t)k * lda + r]) & 0x7FFFFFFFFFFFFFFFull);
  atomicMax(&rowmax[r], m);
}

// Digit slices of A: out[i][r][k] (bf16, K-major, ld ldk, mp rows per slice),
// zero in the padding (r >= n or k >= n).  32 x 32 tiles through shared memory:
// reads along rows of the column-major source, writes along k.
__global__ void oz_slice_a_kernel(int n, int mp, int64_t ldk, const double* __restrict__ A, int64_t lda,
                                  const unsigned long long* __restrict__ rowmax, int* __restrict__ row_exp,
                                  __nv_bfloat16* __restrict__ out)
{
  __shared__ double tile[32][33];
  __shared__ int sexp[32];
  const int r0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;          // 32 x 8
  if (ty == 0) {
    const int r = r0 + tx;
    const int e = r < n ? bound_exponent(rowmax[r]) : 0;
    sexp[tx] = e;
    if (r < mp && blockIdx.y == 0) row_exp[r] = e;
  }
  for (int yy = ty; yy < 32; yy += 8) {
    const int r = r0 + tx, k = k0 + yy;
    tile[tx][yy] = (r < n && k < n) ? A[(int64_t)k * lda + r] : 0.0;
  }
  __syncthreads();
  for (int yy = ty; yy < 32; yy += 8) {
    const int r = r0 + yy, k = k0 + tx;
    if (r >= mp || k >= ldk) continue;
    const double v = tile[yy][tx];
    bool neg = false;
    const unsigned long long F = isfinite(v) ? fixed56(v, sexp[yy], &neg) : 0ull;
#pragma unroll
    for (int i = 0; i < OZ_SLICES; ++i) out[((int64_t)i * mp + r) * ldk + k] = digit_bf16(F, neg, i);
  }
}

// Column maxima of |X| as bit patterns, nrhs <= 16 columns.
__global__ void oz_col_absmax_kernel(int n, int nrhs, const double* __restrict__ X, int64_t ldx,
                                     unsigned long long* __restrict__ colmax)
{
  const int c = blockIdx.y;
  unsigned long long m = 0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
    m = max(m, (unsigned long long)__double_as_longlong(fabs(X[(int64_t)c * ldx + k])));
  for (int off = 16; off > 0; off >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, off));
  if ((threadIdx.x & 31) == 0 && c < nrhs) atomicMax(&colmax[c], m);
}

// Digit slices of X, stacked for the MMA's B operand: row j * 16 + c holds
// digit j of column c, K-major (ld ldk); zero for c >= nrhs and k >= n.
__global__ void oz_slice_x_kernel(int n, int nrhs, int64_t ldk, const double* __restrict__ X, int64_t ldx,
                                  const unsigned long long* __restrict__ colmax, int* __restrict__ col_exp,
                                  __nv_bfloat16* __restrict__ out)
{
  const int c = blockIdx.y;
  const int e = c < nrhs ? bound_exponent(colmax[c]) : 0;
  if (blockIdx.x == 0 && threadIdx.x == 0) col_exp[c] = e;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < ldk; k += (int64_t)gridDim.x * blockDim.x) {
    const double v = (c < nrhs && k < n) ? X[(int64_t)c * ldx + k] : 0.0;
    bool neg = false;
    const unsigned long long F = isfinite(v) ? fixed56(v, e, &neg) : 0ull;
#pragma unroll
    for (int j = 0; j < OZ_SLICES; ++j) out[(int64_t)(j * OZ_RHS + c) * ldk + k] = digit_bf16(F, neg, j);
  }
}

struct OzParams {
  int n, nrhs, mp;
  int chunks, ch_per_cta;
  const int* row_exp;
  const int* col_exp;
  const unsigned long long* rowmax;      // non-finite rows of A
  const unsigned long long* colmax;      // non-finite columns of X
  double* part;                          // [K range][nrhs][n]: (A X) of this range
  int* err;
  uint64_t limit_ns;
};

__global__ void __launch_bounds__(OZ_THREADS, 1)
oz_product_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, const OzParams p)
{
  extern __shared__ __align__(1024) unsigned char oz_smem_raw[];
  unsigned char* smem = (unsigned char*)(((uintptr_t)oz_smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = (uint64_t*)(smem + OZ_STAGES * OZ_STAGE_BYTES);
  uint64_t* empty = full + OZ_STAGES;
  uint64_t* tfull = empty + OZ_STAGES;
  uint64_t* tempty = tfull + 2;
  uint32_t* tmem_slot = (uint32_t*)(tempty + 2);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int rb = blockIdx.x;
  const int ch0 = blockIdx.y * p.ch_per_cta;
  const int nch = min(p.chunks, ch0 + p.ch_per_cta) - ch0;      // >= 1 (host)
  const int ntiles = OZ_SLICES * nch;
  const uint64_t LIMIT = effective_limit(p.limit_ns);
  auto stages_of = [&](int ch) {
    const int len = min(OZ_CHUNK, p.n - ch * OZ_CHUNK);
    return (len + OZ_KS - 1) / OZ_KS;
  };

  if (threadIdx.x == 0) {
    for (int s = 0; s < OZ_STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&tfull[b], 1);
      mbar_init(&tempty[b], 128);
    }
    fence_barrier_init();
  }
  if (warp == 1) tmem_alloc(tmem_slot, OZ_TMEM_COLS);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      int it = 0;
      bool ok = true;
      for (int t = 0; t < ntiles && ok; ++t) {
        const int i = t / nch, ch = ch0 + t % nch;
        const int ks = stages_of(ch);
        for (int kk = 0; kk < ks; ++kk, ++it) {
          const int s = it % OZ_STAGES;
          const uint32_t ph = (uint32_t)(it / OZ_STAGES) & 1u;
          if (!mbar_wait(&empty[s], ph ^ 1u, p.err, LIMIT)) { ok = false; break; }
          unsigned char* sa = smem + s * OZ_STAGE_BYTES;
          mbar_arrive_expect_tx(&full[s], OZ_STAGE_BYTES);
          const int kc = ch * OZ_CHUNK + kk * OZ_KS;                 // multiple of 64 elements: 128-byte aligned
          tma_load_2d(sa, &tmA, &full[s], kc, i * p.mp + rb * OZ_BM);
          tma_load_2d(sa + OZ_A_STAGE, &tmB, &full[s], kc, 0);
        }
      }
      if (!ok) {
        for (int q = it > OZ_STAGES ? it - OZ_STAGES : 0; q < it; ++q)
          mbar_wait(&full[q % OZ_STAGES], (uint32_t)(q / OZ_STAGES) & 1u, p.err, 100000000ull);
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      const uint32_t idesc = idesc_for(1, OZ_BM, OZ_BN);            // bf16 x bf16 -> f32
      int it = 0, tc = 0;
      bool ok = true;
      for (int t = 0; t < ntiles && ok; ++t) {
        const int ch = ch0 + t % nch;
        const int ks = stages_of(ch);
        const int b = tc & 1;
        const uint32_t tph = (uint32_t)(tc >> 1) & 1u;
        if (!mbar_wait(&tempty[b], tph ^ 1u, p.err, LIMIT)) { ok = false; break; }
        tc_fence_after();
        const uint32_t d = tmem_base + (uint32_t)(b * OZ_BN);
        for (int kk = 0; kk < ks; ++kk, ++it) {
          const int s = it % OZ_STAGES;
          const uint32_t ph = (uint32_t)(it / OZ_STAGES) & 1u;
          if (!mbar_wait(&full[s], ph, p.err, LIMIT)) { ok = false; break; }
          tc_fence_after();
          const uint32_t sa = smem_u32(smem + s * OZ_STAGE_BYTES);
          const uint64_t da = sdesc_sw128(sa), db = sdesc_sw128(sa + OZ_A_STAGE);
#pragma unroll
          for (int k4 = 0; k4 < 4; ++k4) {                            // 4 x 16 bf16 of K per stage
            const uint64_t off = (uint64_t)((k4 * 32) >> 4);
            mma_f16(d, da + off, db + off, idesc, (kk > 0 || k4 > 0) ? 1u : 0u);
          }
          mma_commit(&empty[s]);
        }
        if (!ok) break;
        mma_commit(&tfull[b]);
        ++tc;
      }
      if (tc > 0) {
        const int b = (tc - 1) & 1;
        mbar_wait(&tfull[b], (uint32_t)((tc - 1) >> 1) & 1u, p.err, 100000000ull);
      }
    }
  } else {
    const int q = warp & 3;
    const int row = rb * OZ_BM + 32 * q + lane;
    int acc[OZ_SLICES][OZ_RHS];
    double res[OZ_RHS];
#pragma unroll
    for (int c = 0; c < OZ_RHS; ++c) {
      res[c] = 0.0;
#pragma unroll
      for (int j = 0; j < OZ_SLICES; ++j) acc[j][c] = 0;
    }
    bool ok_all = true;
    for (int t = 0; t < ntiles; ++t) {
      const int i = t / nch;
      const bool last = (t % nch) == nch - 1;
      const int b = t & 1;
      const uint32_t tph = (uint32_t)(t >> 1) & 1u;
      int ok = 1;
      if (lane == 0) ok = mbar_wait(&tfull[b], tph, p.err, LIMIT) ? 1 : 0;
      ok = __shfl_sync(0xffffffffu, ok, 0);
      if (!ok) { ok_all = false; break; }
      __syncwarp();
      tc_fence_after();
      const uint32_t tbase = tmem_base + ((uint32_t)(32 * q) << 16) + (uint32_t)(b * OZ_BN);
#pragma unroll
      for (int j = 0; j < OZ_SLICES; ++j) {
        float v[16];
        tmem_ld16(tbase + (uint32_t)(j * OZ_RHS), v);
#pragma unroll
        for (int c = 0; c < OZ_RHS; ++c) acc[j][c] += __float2int_rn(v[c]);     // integer-valued: exact
      }
      tc_fence_before();
      mbar_arrive(&tempty[b]);
      if (last) {
        // sum_j acc_j 2^-7j as two exact int64 groups (|acc| < 2^30, shifts <= 21 bits)
#pragma unroll
        for (int c = 0; c < OZ_RHS; ++c) {
#pragma unroll
          for (int g = 0; g < 2; ++g) {
            long long s = 0;
#pragma unroll
            for (int j = 4 * g; j < 4 * g + 4; ++j) s += (long long)acc[j][c] * (1ll << (OZ_DIGIT * (4 * g + 3 - j)));
            res[c] = fma((double)s, scalbn(1.0, -OZ_DIGIT * (i + 4 * g + 3)), res[c]);
          }
#pragma unroll
          for (int j = 0; j < OZ_SLICES; ++j) acc[j][c] = 0;
        }
      }
    }
    if (ok_all && row < p.n) {
      const int er = p.row_exp[row];
      const bool bad_row = p.rowmax[row] >= kNonFiniteBits;
#pragma unroll
      for (int c = 0; c < OZ_RHS; ++c) {
        if (c < p.nrhs) {
          double v = scalbn(res[c], er + p.col_exp[c] - 2 * OZ_DIGIT);
          if (bad_row || p.colmax[c] >= kNonFiniteBits) v = __longlong_as_double(0x7FF8000000000000ll);
          p.part[((int64_t)blockIdx.y * p.nrhs + c) * p.n + row] = v;
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem_base, OZ_TMEM_COLS);
  }
}

// R = B - sum over K ranges of the partial products (B null: R = A X).
__global__ void oz_reduce_kernel(int n, int nrhs, int splits, const double* __restrict__ part,
                                 const double* __restrict__ B, int64_t ldb, double* __restrict__ R, int64_t ldr)
{
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)n * nrhs) return;
  const int row = (int)(t % n), c = (int)(t / n);
  double s = 0.0;
  for (int k = 0; k < splits; ++k) s += part[((int64_t)k * nrhs + c) * n + row];
  R[(int64_t)c * ldr + row] = B ? B[(int64_t)c * ldb + row] - s : s;
}

inline int cdiv(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }

}  // namespace

int OzakiMatrix::prepare(cudaStream_t s, int n_, const double* A, int64_t lda)
{
  ready = false;
  if (n_ <= 0) return GBS_SUCCESS;
  n = n_;
  mp = cdiv(n, OZ_BM) * OZ_BM;
  ldk = (int64_t)cdiv(n, OZ_KS) * OZ_KS;
  GBS_TRY(slices.reserve(sizeof(__nv_bfloat16) * (size_t)OZ_SLICES * mp * ldk));
  GBS_TRY(rowmax.reserve(sizeof(unsigned long long) * (size_t)mp));
  GBS_TRY(row_exp.reserve(sizeof(int) * (size_t)mp));
  GBS_CUDA_TRY(cudaMemsetAsync(rowmax.p, 0, sizeof(unsigned long long) * (size_t)mp, s));
  PhaseScope ps(s, PH_RESIDUAL, 0.0, 16.0 * (double)n * n + 16.0 * (double)mp * ldk);
  const int rblocks = cdiv(n, 256);
  const int ksplit = std::max(1, std::min(cdiv(n, 64), 4 * device_sm_count() / rblocks));
  const int kspan = cdiv(n, ksplit);
  oz_row_absmax_kernel<<<dim3(rblocks, cdiv(n, kspan)), 256, 0, s>>>(n, A, lda, kspan,
                                                                      rowmax.as<unsigned long long>());
  GBS_CUDA_TRY(cudaGetLastError());
  count_launch();
  const dim3 blk(32, 8), grid2(cdiv(mp, 32), cdiv(ldk, 32));
  oz_slice_a_kernel<<<grid2, blk, 0, s>>>(n, mp, ldk, A, lda, rowmax.as<unsigned long long>(), row_exp.as<int>(),
                                          slices.as<__nv_bfloat16>());
  GBS_CUDA_TRY(cudaGetLastError());
  GBS_TRY(make_tmap(&tmA, slices.p, 2, (int64_t)OZ_SLICES * mp, ldk, ldk, OZ_BM));
  ready = true;
  return GBS_SUCCESS;
}

int ozaki_residual(cudaStream_t s, OzakiMatrix& M, int nrhs, const double* X, int64_t ldx, const double* B,
                   int64_t ldb, double* R, int64_t ldr, OzakiWork& w, int* err)
{
  if (!M.ready) {
    gbs_set_last_message("ozaki_residual: matrix not prepared");
    return GBS_INVALID_ARGUMENT;
  }
  const int n = M.n;
  if (nrhs <= 0) return GBS_SUCCESS;
  if (nrhs > OZ_RHS) {
    gbs_set_last_message("ozaki_residual: at most 16 right-hand sides per call");
    return GBS_INVALID_ARGUMENT;
  }
  const int chunks = cdiv(n, OZ_CHUNK);
  const int tiles_m = M.mp / OZ_BM;
  int splits = std::max(1, std::min(chunks, device_sm_count() / std::max(1, tiles_m)));
  splits = std::max(splits, cdiv(chunks, OZ_MAX_CHUNKS_PER_CTA));
  const int per = cdiv(chunks, splits);
  splits = cdiv(chunks, per);                              // no empty K range
  GBS_TRY(w.xs.reserve(sizeof(__nv_bfloat16) * (size_t)OZ_BN * M.ldk));
  GBS_TRY(w.colmax.reserve(sizeof(unsigned long long) * OZ_RHS));
  GBS_TRY(w.col_exp.reserve(sizeof(int) * OZ_RHS));
  GBS_TRY(w.part.reserve(sizeof(double) * (size_t)splits * nrhs * n));
  static const cudaError_t attr =
      cudaFuncSetAttribute(oz_product_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, OZ_SMEM);
  GBS_CUDA_TRY(attr);
  PhaseScope ps(s, PH_RESIDUAL, 2.0 * n * (double)n * nrhs,
                2.0 * OZ_SLICES * (double)M.mp * M.ldk + 8.0 * (2.0 * n * nrhs + (double)splits * n * nrhs));
  GBS_CUDA_TRY(cudaMemsetAsync(w.colmax.p, 0, sizeof(unsigned long long) * OZ_RHS, s));
  oz_col_absmax_kernel<<<dim3(std::min(cdiv(n, 256), 64), nrhs), 256, 0, s>>>(
      n, nrhs, X, ldx, w.colmax.as<unsigned long long>());
  GBS_CUDA_TRY(cudaGetLastError());
  count_launch();
  oz_slice_x_kernel<<<dim3(std::min(cdiv(M.ldk, 256), 64), OZ_RHS), 256, 0, s>>>(
      n, nrhs, M.ldk, X, ldx, w.colmax.as<unsigned long long>(), w.col_exp.as<int>(), w.xs.as<__nv_bfloat16>());
  GBS_CUDA_TRY(cudaGetLastError());
  count_launch();
  CUtensorMap tmB;
  GBS_TRY(make_tmap(&tmB, w.xs.p, 2, OZ_BN, M.ldk, M.ldk, OZ_BN));
  OzParams p;
  p.n = n;
  p.nrhs = nrhs;
  p.mp = M.mp;
  p.chunks = chunks;
  p.ch_per_cta = per;
  p.row_exp = M.row_exp.as<int>();
  p.col_exp = w.col_exp.as<int>();
  p.rowmax = M.rowmax.as<unsigned long long>();
  p.colmax = w.colmax.as<unsigned long long>();
  p.part = w.part.as<double>();
  p.err = err;
  p.limit_ns = wait_limit_ns();
  oz_product_kernel<<<dim3(tiles_m, splits), OZ_THREADS, OZ_SMEM, s>>>(M.tmA, tmB, p);
  GBS_CUDA_TRY(cudaGetLastError());
  count_launch();
  oz_reduce_kernel<<<cdiv((int64_t)n * nrhs, 256), 256, 0, s>>>(n, nrhs, splits, w.part.as<double>(), B, ldb, R, ldr);
  GBS_CUDA_TRY(cudaGetLastError());
  count_launch();
  return GBS_SUCCESS;
}

}  // namespace gbs
