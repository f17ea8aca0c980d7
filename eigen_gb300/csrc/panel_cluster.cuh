// Panel LU on one thread-block cluster (up to 16 CTAs of 512 threads).
//
// Same arithmetic and pivot rule as panel_lu_kernel (unblocked_lu,
// PartialPivLU.h:365-409; first maximum wins, Visitor.h:173-186), but the
// per-column exchange goes through distributed shared memory and the
// cluster's hardware barrier instead of global scratch and a grid barrier:
//   1. each CTA reduces its rows to one candidate (value, row) and publishes it,
//      with the candidate's row, in its own shared memory (double-buffered by
//      column parity);
//   2. one cluster barrier;
//   3. every CTA reads the C candidates from the other CTAs' shared memory,
//      picks the same winner, and copies the winning row and row j.
// One barrier per column is enough: a CTA rewrites a buffer two columns later,
// after every other CTA has passed the barrier that follows its reads.
// Cluster barriers are hardware barriers over co-scheduled CTAs: no spin loop,
// nothing that can wait forever.
#pragma once

#include <cooperative_groups.h>

#include "dense_kernels.cuh"

namespace gbs {

constexpr int kClusterPanelThreads = 512;
constexpr int kMaxPanelCluster = 16;

template <typename T, int NB>
struct ClusterPanelShared {
  T crow[2][NB];        // this CTA's candidate row
  T rowj[2][NB];        // row j of the panel (held by CTA 0)
  T cval[2];
  int cidx[2];
  T u[NB], oldj[NB];    // winning row and old row j, local copies
  T wval[kClusterPanelThreads / 32];
  int widx[kClusterPanelThreads / 32];
  int win, piv, wrank;
  int spiv[NB];         // the panel's pivots (rows relative to the panel)
};

// a: the panel (m rows, nbc <= NB columns) at row and column k0 of its
// matrix.  map (may be null): the panel's interchanges as a row map (count,
// 256 target rows, 256 source rows; absolute rows) for laswp_gather_kernel.
template <typename T, int NB, int RPT>
__global__ void __launch_bounds__(kClusterPanelThreads)
panel_lu_cluster_kernel(T* __restrict__ a, int64_t lda, int m, int nbc, int k0, int* __restrict__ tr,
                        DeviceStatus* st, int* __restrict__ map)
{
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  const int C = (int)cluster.num_blocks();
  const int rank = (int)cluster.block_rank();
  __shared__ ClusterPanelShared<T, NB> sh;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int g = rank * kClusterPanelThreads + tid;
  const int G = C * kClusterPanelThreads;

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
    T bs = T(-2);
    int bi = 0x7fffffff;
#pragma unroll
    for (int q = 0; q < RPT; ++q) {
      const int r = g + q * G;
      if (r < m && r >= j) {
        const T x = v[q][j];
        const T s = (r == j) ? ((x != x) ? T(INFINITY) : gbs_abs(x)) : pivot_score(x);
        if (better(s, r, bs, bi)) { bs = s; bi = r; }
      }
    }
    warp_argmax(bs, bi);
    if (lane == 0) { sh.wval[warp] = bs; sh.widx[warp] = bi; }
    __syncthreads();
    if (warp == 0) {
      bs = lane < kClusterPanelThreads / 32 ? sh.wval[lane] : T(-2);
      bi = lane < kClusterPanelThreads / 32 ? sh.widx[lane] : 0x7fffffff;
      warp_argmax(bs, bi);
      if (lane == 0) {
        sh.cval[par] = bs;
        sh.cidx[par] = bi;
        sh.win = bi;
      }
    }
    __syncthreads();
    {
      const int winner = sh.win;
#pragma unroll
      for (int q = 0; q < RPT; ++q) {
        const int r = g + q * G;
        if (r < m && r == winner) {
#pragma unroll
          for (int c = 0; c < NB; ++c) sh.crow[par][c] = v[q][c];
        }
        if (r < m && r == j) {
#pragma unroll
          for (int c = 0; c < NB; ++c) sh.rowj[par][c] = v[q][c];
        }
      }
    }
    cluster.sync();
    if (warp == 0) {
      T s = T(-2);
      int i = 0x7fffffff, cw = 0;
      if (lane < C) {
        const ClusterPanelShared<T, NB>* rs = cluster.map_shared_rank(&sh, lane);
        s = rs->cval[par];
        i = rs->cidx[par];
        cw = lane;
      }
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        const T so = __shfl_xor_sync(0xffffffffu, s, off);
        const int io = __shfl_xor_sync(0xffffffffu, i, off);
        const int co = __shfl_xor_sync(0xffffffffu, cw, off);
        if (better(so, io, s, i)) { s = so; i = io; cw = co; }
      }
      if (lane == 0) { sh.piv = i; sh.wrank = cw; }
    }
    __syncthreads();
    if (tid < NB) {
      sh.u[tid] = cluster.map_shared_rank(&sh, sh.wrank)->crow[par][tid];
      sh.oldj[tid] = cluster.map_shared_rank(&sh, 0)->rowj[par][tid];
    }
    __syncthreads();
    const int p = sh.piv;
    const T piv = sh.u[j];
    const bool nz = (piv != T(0));   // biggest_in_corner != 0 (NaN counts as nonzero)
    if (tid == 0) sh.spiv[j] = p;
    if (rank == 0 && tid == 0) {
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
          for (int c = 0; c < NB; ++c) v[q][c] = sh.u[c];
        } else if (r == p) {
#pragma unroll
          for (int c = 0; c < NB; ++c) v[q][c] = sh.oldj[c];
        }
      }
      if (r > j) {
        if (nz) v[q][j] = v[q][j] / piv;
        const T l = v[q][j];
#pragma unroll
        for (int c = j + 1; c < NB; ++c) v[q][c] = fma(-l, sh.u[c], v[q][c]);
      }
    }
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

  // the panel's interchanges as a row map for laswp_gather_kernel: targets
  // are the panel's rows and the pivot rows below them; the source of a target
  // runs the transpositions backwards (the row that ends up there).  Unused
  // slots repeat target 0, so the map always has 2 NB entries.
  if (map && rank == 0) {
    __syncthreads();
    if (tid < 2 * NB) {
      int row = -1;
      if (tid < nbc) row = tid;
      else if (tid >= NB && tid - NB < nbc && sh.spiv[tid - NB] >= nbc) row = sh.spiv[tid - NB];
      if (row < 0) row = 0;
      int pos = row;
      for (int jj = nbc - 1; jj >= 0; --jj) {
        const int pj = sh.spiv[jj];
        if (pos == jj) pos = pj;
        else if (pos == pj) pos = jj;
      }
      map[1 + tid] = k0 + row;
      map[257 + tid] = k0 + pos;
      if (tid == 0) map[0] = 2 * NB;
    }
  }
  cluster.sync();      // no CTA leaves while another may still read its shared memory
}

}  // namespace gbs
