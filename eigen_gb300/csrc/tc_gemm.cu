// tcgen05 trailing-update GEMM (see tc_gemm.cuh).
//
// Kernel layout (one CTA per SM, persistent over output tiles of 128 x 256):
//   warp 0      TMA producer: one 128-byte K-slice of A (128 rows) and of B
//               (256 rows) per pipeline stage, 128B-swizzled, 4-stage ring
//   warp 1      TMEM allocator + MMA issuer: 4 x tcgen05.mma (M=128, N=256,
//               32 bytes of K each) per stage, accumulating in TMEM; commits
//               free the smem stage / publish the finished accumulator
//   warps 2-5   epilogue: tcgen05.ld 32 lanes x 16 columns, C -= acc with
//               column-coalesced FP32 loads/stores (lane = row)
// Two TMEM accumulators (2 x 256 columns) let the epilogue of tile i overlap
// the MMAs of tile i+1.  Every wait is bounded (2 s); on expiry the kernel
// sets the status word's timeout flag, waits for its own copies in flight,
// frees TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <mutex>

#include "gbs_common.cuh"
#include "gbs_profile.cuh"
#include "tc_gemm.cuh"
#include "tc_ptx.cuh"

namespace gbs {
namespace {

constexpr int BM = 128;
constexpr int BN = 256;
constexpr int EPI_COLS = 64;                     // C columns per epilogue pass (loads in flight per lane)
constexpr int ATOM = 128;                          // bytes of K per stage (one swizzle atom)
constexpr int STAGES = 4;
constexpr int NUM_THREADS = 192;
constexpr uint32_t TMEM_COLS = 512;
constexpr int A_STAGE = BM * ATOM;                 // 16 KiB
constexpr int B_STAGE = BN * ATOM;                 // 32 KiB
constexpr int STAGE_BYTES = A_STAGE + B_STAGE;
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 + 256;

struct TcParams {
  int M, N, kiters;         // kiters = K slices of ATOM bytes
  int tiles_m, tiles_n;
  float* C;
  int64_t ldc;
  int lower;
  int tf32;                 // 1: kind::tf32, 0: kind::f16
  uint32_t idesc;
  int* err;
  uint64_t limit_ns;        // wait limit of the pipeline's mbarrier waits (0: the default)
};

__device__ __forceinline__ bool skip_tile(const TcParams& p, int tm, int tn)
{
  return p.lower && (tn * BN >= tm * BM + BM);    // tile strictly above the diagonal
}

// L2 prefetch of this warp's 32 rows of C tile t (one 128-byte line per column,
// eight columns per lane), so that the epilogue's reads of C hit L2.
__device__ __forceinline__ void prefetch_c_tile(const TcParams& p, int t, int q, int lane)
{
  const int tm = t % p.tiles_m, tn = t / p.tiles_m;
  if (skip_tile(p, tm, tn)) return;
  const int row0 = tm * BM + 32 * q;
  if (row0 >= p.M) return;
  for (int c = lane; c < BN; c += 32) {
    const int col = tn * BN + c;
    if (col < p.N) asm volatile("prefetch.global.L2 [%0];" ::"l"(p.C + (int64_t)col * p.ldc + row0));
  }
}

__global__ void __launch_bounds__(NUM_THREADS, 1)
tc_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, const TcParams p)
{
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = (uint64_t*)(smem + STAGES * STAGE_BYTES);
  uint64_t* empty = full + STAGES;
  uint64_t* tfull = empty + STAGES;
  uint64_t* tempty = tfull + 2;
  uint32_t* tmem_slot = (uint32_t*)(tempty + 2);

  griddep_launch_dependents();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&tfull[b], 1);
      mbar_init(&tempty[b], 128);
    }
    fence_barrier_init();
  }
  if (warp == 1) tmem_alloc(tmem_slot, TMEM_COLS);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  griddep_wait();                              // the setup above touches no global memory
  const uint32_t tmem_base = *tmem_slot;
  const int num_tiles = p.tiles_m * p.tiles_n;
  const uint64_t LIMIT = effective_limit(p.limit_ns);

  if (warp == 0) {
    if (lane == 0) {
      int it = 0;
      bool ok = true;
      for (int t = blockIdx.x; t < num_tiles && ok; t += gridDim.x) {
        const int tm = t % p.tiles_m, tn = t / p.tiles_m;
        if (skip_tile(p, tm, tn)) continue;
        for (int kk = 0; kk < p.kiters; ++kk, ++it) {
          const int s = it % STAGES;
          const uint32_t ph = (uint32_t)(it / STAGES) & 1u;
          if (!mbar_wait(&empty[s], ph ^ 1u, p.err, LIMIT)) { ok = false; break; }
          unsigned char* sa = smem + s * STAGE_BYTES;
          mbar_arrive_expect_tx(&full[s], STAGE_BYTES);
          const int kcoord = kk * (p.tf32 ? ATOM / 4 : ATOM / 2);
          tma_load_2d(sa, &tmA, &full[s], kcoord, tm * BM);
          tma_load_2d(sa + A_STAGE, &tmB, &full[s], kcoord, tn * BN);
        }
      }
      if (!ok) {
        // wait (bounded) for this CTA's copies still in flight before teardown
        for (int i = it > STAGES ? it - STAGES : 0; i < it; ++i)
          mbar_wait(&full[i % STAGES], (uint32_t)(i / STAGES) & 1u, p.err, 100000000ull);
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      int it = 0, tc = 0;
      bool ok = true;
      for (int t = blockIdx.x; t < num_tiles && ok; t += gridDim.x) {
        const int tm = t % p.tiles_m, tn = t / p.tiles_m;
        if (skip_tile(p, tm, tn)) continue;
        const int b = tc & 1;
        const uint32_t tph = (uint32_t)(tc >> 1) & 1u;
        if (!mbar_wait(&tempty[b], tph ^ 1u, p.err, LIMIT)) { ok = false; break; }
        tc_fence_after();
        const uint32_t d = tmem_base + (uint32_t)(b * BN);
        for (int kk = 0; kk < p.kiters; ++kk, ++it) {
          const int s = it % STAGES;
          const uint32_t ph = (uint32_t)(it / STAGES) & 1u;
          if (!mbar_wait(&full[s], ph, p.err, LIMIT)) { ok = false; break; }
          tc_fence_after();
          const uint32_t sa = smem_u32(smem + s * STAGE_BYTES);
          const uint64_t da = sdesc_sw128(sa), db = sdesc_sw128(sa + A_STAGE);
#pragma unroll
          for (int k4 = 0; k4 < 4; ++k4) {      // 4 x 32 bytes of K per 128-byte slice
            const uint64_t off = (uint64_t)((k4 * 32) >> 4);
            const uint32_t acc = (kk > 0 || k4 > 0) ? 1u : 0u;
            if (p.tf32) mma_tf32(d, da + off, db + off, p.idesc, acc);
            else mma_f16(d, da + off, db + off, p.idesc, acc);
          }
          mma_commit(&empty[s]);
        }
        if (!ok) break;
        mma_commit(&tfull[b]);
        ++tc;
      }
      if (tc > 0) {
        // the last accumulator must be complete before TMEM is released
        const int b = (tc - 1) & 1;
        mbar_wait(&tfull[b], (uint32_t)((tc - 1) >> 1) & 1u, p.err, 100000000ull);
      }
    }
  } else {
    const int q = warp & 3;                 // TMEM lane quadrant of this warp
    int tc = 0;
    if (blockIdx.x < num_tiles) prefetch_c_tile(p, blockIdx.x, q, lane);
    for (int t = blockIdx.x; t < num_tiles; t += gridDim.x) {
      const int tm = t % p.tiles_m, tn = t / p.tiles_m;
      if (skip_tile(p, tm, tn)) continue;
      // the next tile's C streams into L2 while this tile's accumulator completes
      if (t + (int)gridDim.x < num_tiles) prefetch_c_tile(p, t + (int)gridDim.x, q, lane);
      const int b = tc & 1;
      const uint32_t tph = (uint32_t)(tc >> 1) & 1u;
      // one lane waits, the warp follows: tcgen05.ld below is .sync.aligned
      int ok = 1;
      if (lane == 0) ok = mbar_wait(&tfull[b], tph, p.err, LIMIT) ? 1 : 0;
      ok = __shfl_sync(0xffffffffu, ok, 0);
      if (!ok) break;
      __syncwarp();
      tc_fence_after();
      const int row = tm * BM + 32 * q + lane;
      const bool row_ok = row < p.M;
      const uint32_t tbase = tmem_base + ((uint32_t)(32 * q) << 16) + (uint32_t)(b * BN);
      // C -= acc in two halves of EPI_COLS columns: each lane first issues the
      // loads of its row's EPI_COLS old values (one coalesced 128-byte line per
      // column and warp), so the read-modify-write of C runs with many loads in
      // flight instead of one chunk of 16 at a time
      for (int h = 0; h < BN; h += EPI_COLS) {
        float old[EPI_COLS];
        const int colh = tn * BN + h;
        float* cp = p.C + (int64_t)colh * p.ldc + row;
        {
          const float* lp = cp;
#pragma unroll
          for (int j = 0; j < EPI_COLS; ++j) {
            const int col = colh + j;
            const bool ok = row_ok && col < p.N && (!p.lower || row >= col);
            old[j] = ok ? *lp : 0.f;
            lp += p.ldc;
          }
        }
#pragma unroll
        for (int c = 0; c < EPI_COLS; c += 16) {
          float v[16];
          tmem_ld16(tbase + (uint32_t)(h + c), v);
          float* sp = cp + (int64_t)c * p.ldc;
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const int col = colh + c + j;
            if (row_ok && col < p.N && (!p.lower || row >= col)) *sp = old[c + j] - v[j];
            sp += p.ldc;
          }
        }
      }
      tc_fence_before();
      mbar_arrive(&tempty[b]);
      ++tc;
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem_base, TMEM_COLS);
  }
}

// ------------------------------------------------------------------ packing
__device__ __forceinline__ float round_tf32(float x)
{
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

struct PackJob {
  const float* src;
  int64_t rs, cs;
  int R;
  int pattern;
};

// out[r * ldk + blk * K + k] (K-major) from src(r, k) = src[r*rs + k*cs],
// r < R, k < K, converted to the tier's type; x3 tiers write three K-blocks
// per row, `pattern` selecting hi (0) or lo (1) for each block.  Zero padding
// from nblk K up to Kp.  One CTA per (32-row tile, 32-wide slice of the
// source K): blockIdx.x runs over the tiles of A (the first tiles_a) and then
// of B, blockIdx.y over the K slices (striding when K has more slices than
// the grid).  Each slice is staged in shared memory (loads along the source's
// unit stride), each element read once and written to every block; the CTAs
// with blockIdx.y == 0 also write the padding.
template <typename TO>
__global__ void __launch_bounds__(256)
pack_pair_kernel(PackJob a, PackJob b, int tiles_a, int K, int Kp, TO* __restrict__ outa, TO* __restrict__ outb,
                 int64_t ldk, int kind)
{
  griddep_launch_dependents();
  griddep_wait();
  __shared__ float tile[32][33];
  const bool on_b = (int)blockIdx.x >= tiles_a;
  const PackJob j = on_b ? b : a;
  TO* __restrict__ out = on_b ? outb : outa;
  const int r0 = (on_b ? (int)blockIdx.x - tiles_a : (int)blockIdx.x) * 32;
  if (r0 >= j.R) return;                     // uniform over the CTA
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;   // 32 x 8
  const int nblk = (kind == TC_TF32X3) ? 3 : 1;
  const int Kt = K * nblk;
  for (int k0 = blockIdx.y * 32; k0 < K; k0 += gridDim.y * 32) {
    for (int yy = ty; yy < 32; yy += 8) {
      int r, k;
      if (j.rs == 1) { r = r0 + tx; k = k0 + yy; }
      else { r = r0 + yy; k = k0 + tx; }
      const float v = (r < j.R && k < K) ? j.src[(int64_t)r * j.rs + (int64_t)k * j.cs] : 0.f;
      if (j.rs == 1) tile[tx][yy] = v;
      else tile[yy][tx] = v;
    }
    __syncthreads();
    for (int yy = ty; yy < 32; yy += 8) {
      const int r = r0 + yy, k = k0 + tx;
      if (r >= j.R || k >= K) continue;
      const float v = tile[yy][tx];
      TO* orow = out + (int64_t)r * ldk + k;
      if (kind == TC_TF32X3) {
        const float hi = round_tf32(v);
        const float lo = round_tf32(v - hi);
#pragma unroll
        for (int blk = 0; blk < 3; ++blk) ((float*)orow)[blk * K] = ((j.pattern >> blk) & 1) ? lo : hi;
      } else if constexpr (sizeof(TO) == 4) {
        *orow = kind == TC_TF32 ? round_tf32(v) : v;
      } else if (kind == TC_BF16) {
        *(__nv_bfloat16*)orow = __float2bfloat16_rn(v);
      } else {
        *(__half*)orow = __float2half_rn(v);
      }
    }
    __syncthreads();
  }
  if (blockIdx.y != 0) return;
  const int pad = Kp - Kt;
  for (int e = threadIdx.x; e < 32 * pad; e += blockDim.x) {
    const int r = r0 + e / pad, k = Kt + e % pad;
    if (r < j.R) out[(int64_t)r * ldk + k] = (TO)0.f;
  }
}

// ------------------------------------------------------------------ host
}  // namespace

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn()
{
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)p;
  });
  return fn;
}

int make_tmap(CUtensorMap* tm, const void* base, int esize, int64_t rows, int64_t kp, int64_t ldk, int box_rows)
{
  EncodeTiledFn enc = encode_fn();
  if (!enc) {
    gbs_set_last_message("cuTensorMapEncodeTiled unavailable");
    return GBS_CUDA_ERROR;
  }
  CUtensorMapDataType dt = esize == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_UINT16;
  cuuint64_t dims[2] = {(cuuint64_t)kp, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)(ldk * esize)};
  cuuint32_t box[2] = {(cuuint32_t)(ATOM / esize), (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = enc(tm, dt, 2, const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                   CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    gbs_set_last_message("cuTensorMapEncodeTiled failed");
    return GBS_CUDA_ERROR;
  }
  return GBS_SUCCESS;
}


int tc_gemm_sub(cudaStream_t s, int kind, int M, int N, int K, const float* A, int64_t a_rs, int64_t a_cs,
                const float* B, int64_t b_rs, int64_t b_cs, float* C, int64_t ldc, int lower, DeviceStatus* st,
                TcWorkspace& ws, int max_ctas)
{
  if (M <= 0 || N <= 0 || K <= 0) return GBS_SUCCESS;
  if (kind < TC_BF16 || kind > TC_TF32X3) return GBS_INVALID_ARGUMENT;
  const int esize = (kind == TC_TF32 || kind == TC_TF32X3) ? 4 : 2;
  const int atom_elems = ATOM / esize;
  const int Kt = K * (kind == TC_TF32X3 ? 3 : 1);
  const int Kp = (Kt + atom_elems - 1) / atom_elems * atom_elems;
  const int64_t ldk = Kp;                        // rows 128-byte multiples: TMA strides 16-byte aligned
  GBS_TRY(ws.ak.reserve((size_t)M * ldk * esize));
  GBS_TRY(ws.bk.reserve((size_t)N * ldk * esize));
  {
    PhaseScope ps(s, PH_COPY, 0.0, (double)(M + N) * (4.0 * K + esize * (double)Kp));
    const int tiles_a = (M + 31) / 32, grid = tiles_a + (N + 31) / 32;
    // x3 pattern bits (block -> lo?): A = [hi, hi, lo] (0b100), B = [hi, lo, hi] (0b010)
    const PackJob ja{A, a_rs, a_cs, M, esize == 4 ? 4 : 0}, jb{B, b_cs, b_rs, N, esize == 4 ? 2 : 0};
    const dim3 g2(grid, std::min((K + 31) / 32, 65535));
    if (esize == 4)
      GBS_CUDA_TRY(launch_pdl(pack_pair_kernel<float>, g2, dim3(256), 0, s, ja, jb, tiles_a, K, Kp,
                              ws.ak.as<float>(), ws.bk.as<float>(), ldk, kind));
    else
      GBS_CUDA_TRY(launch_pdl(pack_pair_kernel<uint16_t>, g2, dim3(256), 0, s, ja, jb, tiles_a, K, Kp,
                              ws.ak.as<uint16_t>(), ws.bk.as<uint16_t>(), ldk, kind));
  }
  CUtensorMap tmA, tmB;
  GBS_TRY(make_tmap(&tmA, ws.ak.p, esize, M, Kp, ldk, BM));
  GBS_TRY(make_tmap(&tmB, ws.bk.p, esize, N, Kp, ldk, BN));
  static const cudaError_t attr =
      cudaFuncSetAttribute(tc_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
  GBS_CUDA_TRY(attr);
  TcParams p;
  p.M = M;
  p.N = N;
  p.kiters = Kp / atom_elems;
  p.tiles_m = (M + BM - 1) / BM;
  p.tiles_n = (N + BN - 1) / BN;
  p.C = C;
  p.ldc = ldc;
  p.lower = lower;
  p.tf32 = esize == 4;
  p.idesc = idesc_for(kind == TC_BF16 ? 1 : kind == TC_FP16 ? 0 : 2, BM, BN);
  p.err = &st->timeout;
  p.limit_ns = wait_limit_ns();
  const int tiles = p.tiles_m * p.tiles_n;
  // persistent CTAs, one per SM; max_ctas > 0 leaves the other SMs to work on another stream
  const int ctas = max_ctas > 0 ? std::min(max_ctas, device_sm_count()) : device_sm_count();
  const int grid = tiles < ctas ? tiles : ctas;
  // algorithmic flops of the update (a 3xTF32 update issues three such products on the tensor cores)
  const double flops = 2.0 * M * (double)N * K * (lower ? 0.5 : 1.0);
  const double bytes = 8.0 * M * (double)N * (lower ? 0.5 : 1.0) + (double)(M + N) * Kp * esize;
  PhaseScope ps(s, PH_TC_GEMM, flops, bytes);
  GBS_CUDA_TRY(launch_pdl(tc_gemm_kernel, dim3(grid), dim3(NUM_THREADS), SMEM_BYTES, s, tmA, tmB, p));
  return GBS_SUCCESS;
}

}  // namespace gbs
