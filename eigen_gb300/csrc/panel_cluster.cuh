// Panel LU on one thread-block cluster (up to 16 CTAs of 512 threads).
//
// Same arithmetic and pivot rule as panel_lu_kernel (unblocked_lu,
// PartialPivLU.h:365-409; first maximum wins, Visitor.h:173-186), but the
// per-column exchange goes through distributed shared memory and the
// cluster's hardware barrier instead of global scratch and a grid barrier:
//   1. each CTA reduces its rows to one candidate (value, row);
//   2. it pushes the candidate and the candidate's row (CTA 0 also row j) into
//      every CTA's shared memory (double-buffered by column parity), then one
//      cluster barrier;
//   3. every CTA picks the same winner from its local copies: no remote reads
//      on the critical path.
// One barrier per column is enough: a slot is rewritten two columns later,
// after its reader has passed the barrier that follows its reads.
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
  T crows[2][kMaxPanelCluster][NB];   // every CTA's candidate row, pushed by its owner
  T cval[2][kMaxPanelCluster];
  int cidx[2][kMaxPanelCluster];
  T rowj[2][NB];                      // row j of the panel, pushed by CTA 0
  T mine[NB], minej[NB];              // this CTA's candidate row and row j, staged for the push
  T wval[kClusterPanelThreads / 32];
  int widx[kClusterPanelThreads / 32];
  int spiv[NB];                       // the panel's pivots (rows relative to the panel)
  int tgt[2 * NB], src[2 * NB];       // the interchanges as (target row, source row), relative
  T l11[NB][NB + 1];                  // unit-lower L11 of the panel (CTA 0, for the fused TRSM)
};

// a: the panel (m rows, nbc <= NB columns) at row and column k0 of its
// matrix.  map (may be null): the panel's interchanges as a row map (count,
// 256 target rows, 256 source rows; absolute rows) for laswp_gather_kernel.
// trsm_cols > 0 (needs nbc == NB): CTA 0 also applies the interchanges to the
// trsm_cols columns right of the panel and replaces their top NB rows by
// L11^-1 times them (the U12 block row); the caller leaves those columns out
// of the gather.
template <typename T, int NB, int RPT>
__global__ void __launch_bounds__(kClusterPanelThreads)
panel_lu_cluster_kernel(T* __restrict__ a, int64_t lda, int m, int nbc, int k0, int* __restrict__ tr,
                        DeviceStatus* st, int* __restrict__ map, int trsm_cols)
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
    // 1. this CTA's candidate: first max of |a(r, j)|, r >= j
    T bs = T(-2);
    int bi = 0x7fffffff;
#pragma unroll
    for (int q = 0; q < RPT; ++q) {
      const int r = g + q * G;
      if (r < m && r >= j) {
        const T x = v[q][j];
        const T sc = (r == j) ? ((x != x) ? T(INFINITY) : gbs_abs(x)) : pivot_score(x);
        if (better(sc, r, bs, bi)) { bs = sc; bi = r; }
      }
    }
    warp_argmax(bs, bi);
    if (lane == 0) { sh.wval[warp] = bs; sh.widx[warp] = bi; }
    __syncthreads();
    bs = lane < kClusterPanelThreads / 32 ? sh.wval[lane] : T(-2);     // every warp reduces the same values
    bi = lane < kClusterPanelThreads / 32 ? sh.widx[lane] : 0x7fffffff;
    warp_argmax(bs, bi);
    bs = __shfl_sync(0xffffffffu, bs, 0);
    bi = __shfl_sync(0xffffffffu, bi, 0);
#pragma unroll
    for (int q = 0; q < RPT; ++q) {
      const int r = g + q * G;
      if (r < m && r == bi) {
#pragma unroll
        for (int c = 0; c < NB; ++c) sh.mine[c] = v[q][c];
      }
      if (r < m && r == j) {
#pragma unroll
        for (int c = 0; c < NB; ++c) sh.minej[c] = v[q][c];
      }
    }
    __syncthreads();
    // 2. push the candidate (and, from CTA 0, row j) into every CTA's shared memory
    for (int e = tid; e < C * NB; e += kClusterPanelThreads) {
      const int d = e / NB, c = e % NB;
      ClusterPanelShared<T, NB>* rs = cluster.map_shared_rank(&sh, d);
      rs->crows[par][rank][c] = sh.mine[c];
      if (rank == 0) rs->rowj[par][c] = sh.minej[c];
      if (c == 0) {
        rs->cval[par][rank] = bs;
        rs->cidx[par][rank] = bi;
      }
    }
    cluster.sync();
    // 3. every warp picks the same winner from the local copies
    T s = lane < C ? sh.cval[par][lane] : T(-2);
    int i = lane < C ? sh.cidx[par][lane] : 0x7fffffff;
    int cw = lane;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const T so = __shfl_xor_sync(0xffffffffu, s, off);
      const int io = __shfl_xor_sync(0xffffffffu, i, off);
      const int co = __shfl_xor_sync(0xffffffffu, cw, off);
      if (better(so, io, s, i)) { s = so; i = io; cw = co; }
    }
    const int p = __shfl_sync(0xffffffffu, i, 0);
    const int wr = __shfl_sync(0xffffffffu, cw, 0);
    const T* u = sh.crows[par][wr];
    const T* oldj = sh.rowj[par];
    const T piv = u[j];
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
          for (int c = 0; c < NB; ++c) v[q][c] = u[c];
        } else if (r == p) {
#pragma unroll
          for (int c = 0; c < NB; ++c) v[q][c] = oldj[c];
        }
      }
      if (r > j) {
        if (nz) v[q][j] = v[q][j] / piv;
        const T l = v[q][j];
#pragma unroll
        for (int c = j + 1; c < NB; ++c) v[q][c] = fma(-l, u[c], v[q][c]);
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

  // the panel's interchanges as (target, source) rows: targets are the
  // panel's rows and the pivot rows below them; the source of a target runs
  // the transpositions backwards (the row that ends up there).  Unused slots
  // repeat target 0, so the map always has 2 NB entries.
  if (rank == 0 && (map || trsm_cols > 0)) {
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
      sh.tgt[tid] = row;
      sh.src[tid] = pos;
      if (map) {
        map[1 + tid] = k0 + row;
        map[257 + tid] = k0 + pos;
        if (tid == 0) map[0] = 2 * NB;
      }
    }
    if (trsm_cols > 0) {
      if (tid < NB) {                          // L11 from the rows this CTA holds (rows 0..NB-1, slot 0)
#pragma unroll
        for (int c = 0; c < NB; ++c) sh.l11[tid][c] = v[0][c];
      }
      __syncthreads();
      // interchanges on the trsm_cols columns, one warp per column
      constexpr int Q = (2 * NB + 31) / 32;
      for (int cc = warp; cc < trsm_cols; cc += kClusterPanelThreads / 32) {
        T* col = a + (int64_t)(nbc + cc) * lda;
        T val[Q];
#pragma unroll
        for (int q = 0; q < Q; ++q) {
          const int t = lane + 32 * q;
          val[q] = t < 2 * NB ? col[sh.src[t]] : T(0);
        }
        __syncwarp();
#pragma unroll
        for (int q = 0; q < Q; ++q) {
          const int t = lane + 32 * q;
          if (t < 2 * NB) col[sh.tgt[t]] = val[q];
        }
      }
      __syncthreads();
      // U12 = L11^-1 A12 (unit lower), one column per thread
      for (int cc = tid; cc < trsm_cols; cc += kClusterPanelThreads) {
        T* col = a + (int64_t)(nbc + cc) * lda;
        T x[NB];
#pragma unroll
        for (int jj = 0; jj < NB; ++jj) x[jj] = col[jj];
#pragma unroll
        for (int jj = 0; jj < NB; ++jj) {
          asm volatile("" ::: "memory");     // keep each step's L11 loads next to their use (register pressure)
#pragma unroll
          for (int ii = jj + 1; ii < NB; ++ii) x[ii] = fma(-sh.l11[ii][jj], x[jj], x[ii]);
        }
#pragma unroll
        for (int jj = 0; jj < NB; ++jj) col[jj] = x[jj];
      }
    }
  }
  cluster.sync();      // no CTA leaves while another may still read its shared memory
}

}  // namespace gbs
