#pragma once
// Panel factorization of the plain LU path (one translation unit per scalar
// type, so the unrolled register kernels compile in parallel).
#include <algorithm>

#include "dense_driver.cuh"
#include "dense_kernels.cuh"
#include "gbs_profile.cuh"

namespace gbs {

static inline int ceil_div(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }


template <typename T, int RPT>
static int launch_panel(cudaStream_t s, T* a, int64_t lda, int m, int nbc, int k0, int* tr, DevBuf& scratch,
                        DeviceStatus* st, int P)
{
  void* sp = scratch.p;
  PhaseScope ps(s, PH_PANEL, (double)m * nbc * nbc, sizeof(T) * 2.0 * m * nbc);
  void* args[] = {&a, &lda, &m, &nbc, &k0, &tr, &sp, &st};
  GBS_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)panel_lu_kernel<T, kPanelNB, RPT>, dim3(P),
                                           dim3(kPanelThreads), args, 0, s));
  return GBS_SUCCESS;
}

template <typename T, int RPT>
static int panel_capacity()
{
  static int cap = -1;
  if (cap < 0) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, panel_lu_kernel<T, kPanelNB, RPT>, kPanelThreads, 0);
    cap = per_sm * device_sm_count();
  }
  return cap;
}

template <typename T>
int panel_factor(cudaStream_t s, T* a, int64_t lda, int m, int nbc, int k0, int* tr, DevBuf& scratch,
                        DeviceStatus* st)
{
  // rows per thread: smallest power of two that keeps the grid co-resident
  // and below one CTA per SM (fewer CTAs make the per-column barrier cheaper)
  const int sms = device_sm_count();
  int rpt = 1;
  int P = ceil_div(m, kPanelThreads * rpt);
  while (P > sms && rpt < 2) { rpt *= 2; P = ceil_div(m, kPanelThreads * rpt); }
  int cap = rpt == 1 ? panel_capacity<T, 1>() : panel_capacity<T, 2>();
  if (P > cap) {
    gbs_set_last_message("panel too tall for one cooperative launch");
    return GBS_INVALID_ARGUMENT;
  }
  GBS_TRY(scratch.reserve(panel_scratch_bytes<T, kPanelNB>(P)));
  if (rpt == 1) return launch_panel<T, 1>(s, a, lda, m, nbc, k0, tr, scratch, st, P);
  return launch_panel<T, 2>(s, a, lda, m, nbc, k0, tr, scratch, st, P);
}

}  // namespace gbs
