#pragma once
// Panel factorization of the plain LU path (one translation unit per scalar
// type, so the unrolled register kernels compile in parallel).
#include <algorithm>

#include "dense_driver.cuh"
#include "dense_kernels.cuh"
#include "gbs_profile.cuh"
#include "panel_cluster.cuh"

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
  static const int cap = [] {                  // once per process (thread-safe static initialisation)
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, panel_lu_kernel<T, kPanelNB, RPT>, kPanelThreads, 0);
    return per_sm * device_sm_count();
  }();
  return cap;
}

// Largest cluster (power of two, <= 16) the device schedules for this kernel.
template <typename T, int RPT>
static int cluster_panel_limit()
{
  static const int limit = [] {                // once per process (thread-safe static initialisation)
    int lim = 0;
    const void* k = (const void*)panel_lu_cluster_kernel<T, kPanelNB, RPT>;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) cudaGetLastError();
    const int dyn = (int)cluster_panel_dyn_smem<T, kPanelNB, RPT>();
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn) != cudaSuccess) {
      cudaGetLastError();
      return 0;                                // no cluster panel: the cooperative kernel takes every panel
    }
    for (int c = kMaxPanelCluster; c >= 1 && lim == 0; c /= 2) {
      cudaLaunchConfig_t cfg = {};
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = c;
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      cfg.gridDim = dim3(c);
      cfg.blockDim = dim3(kClusterPanelThreads);
      cfg.dynamicSmemBytes = dyn;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      int nclusters = 0;
      if (cudaOccupancyMaxActiveClusters(&nclusters, k, &cfg) == cudaSuccess && nclusters > 0) lim = c;
      else cudaGetLastError();
    }
    return lim;
  }();
  return limit;
}

template <typename T, int RPT>
static int launch_cluster_panel(cudaStream_t s, T* a, int64_t lda, int m, int nbc, int k0, int* tr,
                                DeviceStatus* st, int C, int* map, int trsm_cols)
{
  PhaseScope ps(s, PH_PANEL, (double)m * nbc * nbc, sizeof(T) * 2.0 * m * nbc);
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute at[2];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = C;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  at[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;   // the kernel waits at entry (griddep_wait)
  at[1].val.programmaticStreamSerializationAllowed = 1;
  cfg.gridDim = dim3(C);
  cfg.blockDim = dim3(kClusterPanelThreads);
  cfg.dynamicSmemBytes = cluster_panel_dyn_smem<T, kPanelNB, RPT>();
  cfg.stream = s;
  cfg.attrs = at;
  cfg.numAttrs = 2;
  GBS_CUDA_TRY(cudaLaunchKernelEx(&cfg, panel_lu_cluster_kernel<T, kPanelNB, RPT>, a, lda, m, nbc, k0, tr, st, map,
                                  trsm_cols));
  return GBS_SUCCESS;
}

// Largest cluster (power of two, <= 16) the device schedules for the
// tournament-pivoting kernel.
template <typename T>
static int tournament_panel_limit()
{
  static const int limit = [] {
    int lim = 0;
    const void* k = (const void*)panel_lu_tournament_kernel<T, kPanelNB>;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) cudaGetLastError();
    const int dyn = (int)tournament_dyn_smem<T, kPanelNB>();
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn) != cudaSuccess) {
      cudaGetLastError();
      return 0;
    }
    for (int c = kMaxPanelCluster; c >= 2 && lim == 0; c /= 2) {
      cudaLaunchConfig_t cfg = {};
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = c;
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      cfg.gridDim = dim3(c);
      cfg.blockDim = dim3(kClusterPanelThreads);
      cfg.dynamicSmemBytes = dyn;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      int nclusters = 0;
      if (cudaOccupancyMaxActiveClusters(&nclusters, k, &cfg) == cudaSuccess && nclusters > 0) lim = c;
      else cudaGetLastError();
    }
    return lim;
  }();
  return limit;
}

template <typename T>
static int launch_tournament_panel(cudaStream_t s, T* a, int64_t lda, int m, int k0, int* tr, DeviceStatus* st,
                                   int C, int* map, int trsm_cols)
{
  PhaseScope ps(s, PH_PANEL, (double)m * kPanelNB * kPanelNB, sizeof(T) * 2.0 * m * kPanelNB);
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = C;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3(C);
  cfg.blockDim = dim3(kClusterPanelThreads);
  cfg.dynamicSmemBytes = tournament_dyn_smem<T, kPanelNB>();
  cfg.stream = s;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  GBS_CUDA_TRY(cudaLaunchKernelEx(&cfg, panel_lu_tournament_kernel<T, kPanelNB>, a, lda, m, k0, tr, st, map,
                                  trsm_cols));
  return GBS_SUCCESS;
}

// The panel on one cluster when its rows fit (one row per thread, two for
// FP32), else on the cooperative grid kernel.  With map_out, the cluster
// kernel also leaves the panel's interchanges as a row map in scratch and
// *map_out points to it (null after the cooperative kernel).  trsm_cols > 0
// asks the cluster kernel to also interchange and solve (U12 = L11^-1 A12) the
// trsm_cols columns right of the panel; *trsm_done says whether it did.
template <typename T>
int panel_factor(cudaStream_t s, T* a, int64_t lda, int m, int nbc, int k0, int* tr, DevBuf& scratch,
                        DeviceStatus* st, const int** map_out, int trsm_cols, bool* trsm_done, bool tournament)
{
  if (map_out) *map_out = nullptr;
  if (trsm_done) *trsm_done = false;
  if (tournament && nbc == kPanelNB && m > kClusterPanelThreads && m <= kMaxPanelCluster * kClusterPanelThreads) {
    const int C = panel_cluster_ctas(m);
    if (C <= tournament_panel_limit<T>()) {
      int* map = nullptr;
      if (map_out) {
        GBS_TRY(scratch.reserve(sizeof(int) * kLaswpMapInts));
        map = scratch.as<int>();
        *map_out = map;
      }
      const int tc = trsm_done ? trsm_cols : 0;
      if (trsm_done) *trsm_done = tc > 0;
      return launch_tournament_panel<T>(s, a, lda, m, k0, tr, st, C, map, tc);
    }
  }
  {
    constexpr int rpt_max = sizeof(T) == 8 ? 1 : 2;
    int C = 1;
    while (C * kClusterPanelThreads < m && C < kMaxPanelCluster) C *= 2;
    const int rpt = C * kClusterPanelThreads >= m ? 1 : 2;
    if (rpt <= rpt_max && C * kClusterPanelThreads * rpt >= m) {
      const int lim = rpt == 1 ? cluster_panel_limit<T, 1>() : cluster_panel_limit<T, rpt_max>();
      if (C <= lim) {
        int* map = nullptr;
        if (map_out) {
          GBS_TRY(scratch.reserve(sizeof(int) * kLaswpMapInts));
          map = scratch.as<int>();
          *map_out = map;
        }
        const int tc = (trsm_done && nbc == kPanelNB) ? trsm_cols : 0;
        if (trsm_done) *trsm_done = tc > 0;
        if (rpt == 1) return launch_cluster_panel<T, 1>(s, a, lda, m, nbc, k0, tr, st, C, map, tc);
        return launch_cluster_panel<T, rpt_max>(s, a, lda, m, nbc, k0, tr, st, C, map, tc);
      }
    }
  }
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

template <typename T>
int panel_preload()
{
  constexpr int rpt_max = sizeof(T) == 8 ? 1 : 2;
  cudaFuncAttributes fa;
  GBS_CUDA_TRY(cudaFuncGetAttributes(&fa, (const void*)panel_lu_kernel<T, kPanelNB, 1>));
  GBS_CUDA_TRY(cudaFuncGetAttributes(&fa, (const void*)panel_lu_kernel<T, kPanelNB, 2>));
  GBS_CUDA_TRY(cudaFuncGetAttributes(&fa, (const void*)panel_lu_cluster_kernel<T, kPanelNB, 1>));
  GBS_CUDA_TRY(cudaFuncGetAttributes(&fa, (const void*)panel_lu_cluster_kernel<T, kPanelNB, rpt_max>));
  (void)panel_capacity<T, 1>();
  (void)panel_capacity<T, 2>();
  (void)cluster_panel_limit<T, 1>();
  (void)cluster_panel_limit<T, rpt_max>();
  return GBS_SUCCESS;
}

}  // namespace gbs
