// Common device/host utilities of libgb300solve: status codes, error checks,
// the bounded grid barrier used by the cooperative panel kernels, and small
// warp-level helpers.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "gb300solve.h"

#define GBS_CUDA_TRY(expr)                                     \
  do {                                                         \
    cudaError_t _e = (expr);                                   \
    if (_e != cudaSuccess) {                                   \
      gbs_set_last_cuda_error(_e, #expr, __FILE__, __LINE__);  \
      return GBS_CUDA_ERROR;                                   \
    }                                                          \
  } while (0)

#define GBS_TRY(expr)                    \
  do {                                   \
    int _s = (expr);                     \
    if (_s != GBS_SUCCESS) return _s;    \
  } while (0)

void gbs_set_last_cuda_error(cudaError_t e, const char* what, const char* file, int line);
void gbs_set_last_message(const char* msg);

namespace gbs {

// Device-side status word shared by the kernels of one factorization.  Kernels
// that wait on other CTAs give up after a deadline, set `timeout` and return,
// so a stuck wait ends the launch with an error status instead of hanging.
struct DeviceStatus {
  unsigned int bar_count;   // grid barrier arrival counter
  unsigned int bar_gen;     // grid barrier generation
  int timeout;              // set to 1 by any wait that ran out of time
  int info;                 // LLT: first failing column (-1 = none); LU: first zero pivot (-1)
  int nb_transpositions;    // LU: number of actual row swaps
  int pad0;
  unsigned long long limit_ns;  // wait limit of this factorization's spins (0: the default)
};

__device__ __forceinline__ uint64_t globaltimer_ns()
{
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned int ld_acquire_u32(const unsigned int* p)
{
  unsigned int v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Release store at GPU scope: after a CTA barrier, it publishes the writes
// every thread of the CTA made before the barrier (the barrier orders them
// before this store, and release is cumulative).
__device__ __forceinline__ void st_release_u32(unsigned int* p, unsigned int v)
{
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Programmatic dependent launch.  A kernel launched by launch_pdl may be
// scheduled while the previous kernel of its stream still runs: it calls
// griddep_wait() before it reads or writes any global memory, which waits for
// that kernel's completion and the visibility of its writes.  Every kernel
// that may precede one calls griddep_launch_dependents() at entry, so that the
// next kernel's CTAs start their launch and prologue early; that grid is
// scheduled only once every CTA of this one has started, so its waiting CTAs
// never keep this grid's CTAs off the SMs.  Both are no-ops without a
// programmatic dependency.
__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void griddep_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                              Args&&... args)
{
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, static_cast<Args&&>(args)...);
}

__device__ __forceinline__ int ld_volatile_i32(const int* p)
{
  return *(const volatile int*)p;
}

// Default wait limit of every inter-CTA spin in this library (2 s of wall
// time).  The limit in force is a process-wide runtime value
// (gbs_set_wait_limit) that the host passes to each launch; 0 means this default.
constexpr uint64_t kSpinDeadlineNs = 2000000000ull;

// Host: the wait limit the next launches get, in nanoseconds.
uint64_t wait_limit_ns();

__host__ __device__ __forceinline__ uint64_t effective_limit(uint64_t ns) { return ns ? ns : kSpinDeadlineNs; }

// Sense-free grid barrier for a cooperative launch (all CTAs co-resident).
// Returns false (on every thread of the CTA) if the barrier timed out or if
// another CTA already reported a timeout; the caller must then return.
__device__ __forceinline__ bool grid_barrier(DeviceStatus* st, unsigned int nblocks)
{
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    unsigned int gen = ld_acquire_u32(&st->bar_gen);
    __threadfence();
    unsigned int arrived = atomicAdd(&st->bar_count, 1u);
    if (arrived == nblocks - 1) {
      atomicExch(&st->bar_count, 0u);
      __threadfence();
      atomicAdd(&st->bar_gen, 1u);
    } else {
      const uint64_t limit = effective_limit(*(const volatile unsigned long long*)&st->limit_ns);
      uint64_t t0 = globaltimer_ns();
      unsigned int spins = 0;
      while (ld_acquire_u32(&st->bar_gen) == gen) {
        if ((++spins & 63u) == 0) {
          if (ld_volatile_i32(&st->timeout) || globaltimer_ns() - t0 > limit) {
            atomicExch(&st->timeout, 1);
            ok = 0;
            break;
          }
        }
        __nanosleep(20);
      }
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

template <typename T>
__device__ __forceinline__ T gbs_abs(T v) { return v < T(0) ? -v : v; }

// Pivot score of the reference's unblocked LU (PartialPivLU.h:380-382 with
// Visitor.h:173-186): the first maximum of |a| wins; a NaN never wins except
// as the first element of the column, which the caller handles separately.
template <typename T>
__device__ __forceinline__ T pivot_score(T v)
{
  T a = gbs_abs(v);
  return (a != a) ? T(-1) : a;
}

// (score, index) comparison: larger score, then lower index.
template <typename T>
__device__ __forceinline__ bool better(T sa, int ia, T sb, int ib)
{
  return sa > sb || (sa == sb && ia < ib);
}

template <typename T>
__device__ __forceinline__ void warp_argmax(T& s, int& i)
{
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    T so = __shfl_xor_sync(0xffffffffu, s, off);
    int io = __shfl_xor_sync(0xffffffffu, i, off);
    if (better(so, io, s, i)) { s = so; i = io; }
  }
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v)
{
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  return v;
}

template <typename T>
__device__ __forceinline__ T warp_max(T v)
{
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    T o = __shfl_xor_sync(0xffffffffu, v, off);
    v = o > v ? o : v;
  }
  return v;
}

}  // namespace gbs
