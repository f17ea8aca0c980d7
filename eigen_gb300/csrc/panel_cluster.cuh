// Panel LU on one thread-block cluster (up to 16 CTAs of 512 threads).
//
// Same arithmetic and pivot rule as panel_lu_kernel (unblocked_lu,
// PartialPivLU.h:365-409; first maximum wins, Visitor.h:173-186), with the
// per-column exchange through distributed shared memory and the cluster's
// hardware barrier instead of global scratch and a grid barrier.
//
// Layout.  Each thread holds RPT rows of the panel in registers.  At step j a
// row's registers hold its columns j .. NB-1 in slots 0 .. NB-1-j: after the
// rank-1 update of step j every row shifts left by one slot, so the current
// column is always slot 0 and the column loop runs as a plain loop (a small
// body that stays in the instruction cache) instead of NB unrolled copies.
//
// Rows never move.  Each thread-row carries its current position; the
// interchange of step j swaps the positions of the pivot row and the row at
// position j, so the pivot search sees exactly the reference's row order (the
// first maximum is the lowest position) without copying a row between CTAs.
// Finished entries (the row's L part, and its U part once it is a pivot row)
// collect in shared memory and are written once, at the row's final position.
//
// Pivot search on integer keys: an entry x maps to bits(|x|) + 1, which orders
// like |x|, and a NaN to 0 (a NaN is never the first maximum unless it is the
// column's first entry, which maps to the key of +inf, the largest).  The
// largest key, then the lowest position, wins -- the reference's strict '>'
// scan -- in two or three redux.sync instructions per warp.
//
// Per column j:
//   1. every CTA picks the same winner from its local copies of the cluster's
//      candidates (no remote reads on the critical path), scales its rows and
//      updates column j+1 only;
//   2. each CTA reduces its rows to one candidate for column j+1; the owning
//      thread finishes its row's update, and its warp stores row and key into
//      every CTA (one destination CTA per lane, 16-byte stores);
//   3. cluster barrier: the warps that stored remotely arrive with release,
//      the rest relaxed; between arrive and wait every thread applies the
//      rank-1 update to its rows' other columns, off the critical path.
// The candidate slots are triple-buffered by column: a slot is rewritten for
// column j+3, whose writers have passed the barrier of column j+2, which every
// CTA reaches only after its update of column j -- the last read of the slot.
// Cluster barriers are hardware barriers over co-scheduled CTAs: no spin loop,
// nothing that can wait forever.  The status word (swap count, first zero
// pivot) is read once and written once per launch.
#pragma once

#include <cooperative_groups.h>

#include "dense_kernels.cuh"

namespace gbs {

constexpr int kClusterPanelThreads = 512;
constexpr int kMaxPanelCluster = 16;

template <typename T> struct PivotKey;
template <> struct PivotKey<float> { typedef unsigned int type; };
template <> struct PivotKey<double> { typedef unsigned long long type; };

// Integer pivot key of entry x; first: x is the column's first entry (position j).
template <typename T>
__device__ __forceinline__ typename PivotKey<T>::type pivot_key(T x, bool first)
{
  typedef typename PivotKey<T>::type K;
  if (sizeof(T) == 4) {
    if (x != x) return first ? (K)0x7F800001u : (K)0;
    return (K)__float_as_uint(fabsf((float)x)) + (K)1;
  }
  if (x != x) return first ? (K)0x7FF0000000000001ull : (K)0;
  return (K)__double_as_longlong(fabs((double)x)) + (K)1;
}

// Warp-wide (largest key, lowest position); every lane gets the result.
__device__ __forceinline__ void warp_keymax(unsigned int& k, int& i)
{
  const unsigned int km = __reduce_max_sync(0xffffffffu, k);
  i = (int)__reduce_min_sync(0xffffffffu, k == km ? (unsigned int)i : 0x7fffffffu);
  k = km;
}
__device__ __forceinline__ void warp_keymax(unsigned long long& k, int& i)
{
  const unsigned int hi = (unsigned int)(k >> 32), lo = (unsigned int)k;
  const unsigned int hm = __reduce_max_sync(0xffffffffu, hi);
  const unsigned int lm = __reduce_max_sync(0xffffffffu, hi == hm ? lo : 0u);
  const bool top = hi == hm && lo == lm;
  i = (int)__reduce_min_sync(0xffffffffu, top ? (unsigned int)i : 0x7fffffffu);
  k = ((unsigned long long)hm << 32) | lm;
}

__device__ __forceinline__ void cluster_arrive(bool release)
{
  if (release) asm volatile("barrier.cluster.arrive.release.aligned;\n" ::: "memory");
  else asm volatile("barrier.cluster.arrive.relaxed.aligned;\n" ::: "memory");
}

__device__ __forceinline__ void cluster_wait() { asm volatile("barrier.cluster.wait.acquire.aligned;\n" ::: "memory"); }

template <typename T, int NB>
struct ClusterPanelShared {
  typedef typename PivotKey<T>::type K;
  __align__(16) T crows[3][kMaxPanelCluster][NB];   // every CTA's candidate row (slot s = column j + s)
  K ckey[3][kMaxPanelCluster];
  int cidx[3][kMaxPanelCluster];
  __align__(16) T outrow[NB];                       // this CTA's candidate row, staged for the stores
  K wkey[kClusterPanelThreads / 32];
  int widx[kClusterPanelThreads / 32];
  int spiv[NB];                       // the panel's pivots (positions relative to the panel)
  int tgt[2 * NB], src[2 * NB];       // the interchanges as (target row, source row), relative
  T l11[NB][NB + 1];                  // unit-lower L11 of the panel (CTA 0, for the fused TRSM)
};

// Dynamic shared memory of one CTA: the finished entries of its rows,
// fin[c * (threads * RPT) + slot] for column c.
template <typename T, int NB, int RPT>
constexpr size_t cluster_panel_dyn_smem()
{
  return sizeof(T) * (size_t)NB * kClusterPanelThreads * RPT;
}

// This CTA's candidate (largest key, lowest position) from each thread's
// best (bk, bi); every lane of every warp gets it.
template <typename T, int NB>
__device__ __forceinline__ void cluster_panel_cta_candidate(ClusterPanelShared<T, NB>& sh,
                                                            typename PivotKey<T>::type bk, int bi,
                                                            typename PivotKey<T>::type& ck, int& ci)
{
  typedef typename PivotKey<T>::type K;
  constexpr int NW = kClusterPanelThreads / 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  warp_keymax(bk, bi);
  if (lane == 0) { sh.wkey[warp] = bk; sh.widx[warp] = bi; }
  __syncthreads();
  ck = lane < NW ? sh.wkey[lane] : (K)0;
  ci = lane < NW ? sh.widx[lane] : 0x7fffffff;
  warp_keymax(ck, ci);
}

// The owner warp (its row staged in sh.outrow) stores row, key and position
// into slot sl of every CTA; a CTA without a candidate stores an empty one
// from warp 0.  Returns whether this warp stored into other CTAs.
template <typename T, int NB>
__device__ __forceinline__ bool cluster_panel_push(ClusterPanelShared<T, NB>& sh, int sl,
                                                   typename PivotKey<T>::type ck, int ci, bool owner_warp, int C,
                                                   int rank)
{
  namespace cg = cooperative_groups;
  typedef typename PivotKey<T>::type K;
  cg::cluster_group cluster = cg::this_cluster();
  constexpr int CH = NB * (int)sizeof(T) / 16;         // 16-byte chunks of a row
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (ci != 0x7fffffff) {
    if (!owner_warp) return false;
    // (destination, chunk) pairs dealt over the lanes: lane l serves CTA
    // l % C with chunks l / C, l / C + 32 / C, ...
    const int d = lane % C;
    ClusterPanelShared<T, NB>* rs = cluster.map_shared_rank(&sh, d);
    for (int ch = lane / C; ch < CH; ch += 32 / C)
      reinterpret_cast<float4*>(rs->crows[sl][rank])[ch] = reinterpret_cast<const float4*>(sh.outrow)[ch];
    if (lane < C) {
      rs->ckey[sl][rank] = ck;
      rs->cidx[sl][rank] = ci;
    }
    return true;
  }
  if (warp != 0) return false;
  if (lane < C) {
    ClusterPanelShared<T, NB>* rs = cluster.map_shared_rank(&sh, lane);
    rs->ckey[sl][rank] = (K)0;
    rs->cidx[sl][rank] = 0x7fffffff;
  }
  return true;
}

// Rank-1 update of a row's columns j+2.. and the shift by one slot; slot 1
// (column j+1) was updated already.
template <typename T, int NB>
__device__ __forceinline__ void cluster_panel_shift_update(T (&v)[NB], T l, const T* u)
{
  v[0] = v[1];
#pragma unroll
  for (int c = 1; c < NB - 1; ++c) v[c] = fma(-l, u[c + 1], v[c + 1]);
  v[NB - 1] = T(0);
}

// CTA 0's part after the panel's rows are final: the panel's interchanges as
// (target, source) rows into sh.tgt / sh.src (and the row map, when asked),
// then, for trsm_cols > 0, the interchanges and U12 = L11^-1 A12 of the
// trsm_cols columns right of the panel.  sh: any shared layout with spiv, tgt,
// src and l11 members; sh.spiv holds the panel's transpositions.
template <typename T, int NB, typename SH>
__device__ void cluster_panel_tail(SH& sh, T* __restrict__ a, int64_t lda, int m, int nbc, int k0,
                                   int* __restrict__ map, int trsm_cols)
{
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // the panel's interchanges as (target, source) rows: targets are the
  // panel's rows and the pivot rows below them; the source of a target runs
  // the transpositions backwards (the row that ends up there).  Unused slots
  // repeat target 0, so the map always has 2 NB entries.
  {
    __syncthreads();
    if (tid < 2 * NB) {
      int row = -1;
      if (tid < nbc) row = tid;
      else if (tid >= NB && tid - NB < nbc && sh.spiv[tid - NB] >= nbc) row = sh.spiv[tid - NB];
      if (row < 0) row = 0;
      int p = row;
      for (int jj = nbc - 1; jj >= 0; --jj) {
        const int pj = sh.spiv[jj];
        if (p == jj) p = pj;
        else if (p == pj) p = jj;
      }
      sh.tgt[tid] = row;
      sh.src[tid] = p;
      if (map) {
        map[1 + tid] = k0 + row;
        map[257 + tid] = k0 + p;
        if (tid == 0) map[0] = 2 * NB;
      }
    }
    if (trsm_cols > 0) {
      for (int e = tid; e < NB * NB; e += kClusterPanelThreads) {
        const int r = e % NB, c = e / NB;
        sh.l11[r][c] = (r > c && r < m) ? a[(int64_t)c * lda + r] : T(0);
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
}

// a: the panel (m rows, nbc <= NB columns) at row and column k0 of its
// matrix.  map (may be null): the panel's interchanges as a row map (count,
// 256 target rows, 256 source rows; absolute rows) for laswp_gather_kernel.
// trsm_cols > 0 (needs nbc == NB): CTA 0 also applies the interchanges to the
// trsm_cols columns right of the panel and replaces their top NB rows by
// L11^-1 times them (the U12 block row); the caller leaves those columns out
// of the gather.  Dynamic shared memory: cluster_panel_dyn_smem<T, NB, RPT>().
template <typename T, int NB, int RPT>
__global__ void __launch_bounds__(kClusterPanelThreads)
panel_lu_cluster_kernel(T* __restrict__ a, int64_t lda, int m, int nbc, int k0, int* __restrict__ tr,
                        DeviceStatus* st, int* __restrict__ map, int trsm_cols)
{
  static_assert(NB == 32, "one lane per panel column");
  griddep_launch_dependents();
  griddep_wait();
  typedef typename PivotKey<T>::type K;
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  const int C = (int)cluster.num_blocks();
  const int rank = (int)cluster.block_rank();
  __shared__ ClusterPanelShared<T, NB> sh;
  extern __shared__ __align__(16) unsigned char cluster_panel_dyn[];
  T* fin = reinterpret_cast<T*>(cluster_panel_dyn);
  constexpr int S = kClusterPanelThreads * RPT;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int g = rank * kClusterPanelThreads + tid;
  const int G = C * kClusterPanelThreads;
  const bool keeper = rank == 0 && tid == 0;        // keeps the status counters of this launch
  int swaps = 0, first_zero = -1;

  T v[RPT][NB];
  int pos[RPT];
#pragma unroll
  for (int q = 0; q < RPT; ++q) {
    const int r = g + q * G;
    pos[q] = r;
#pragma unroll
    for (int c = 0; c < NB; ++c) v[q][c] = (r < m && c < nbc) ? a[(int64_t)c * lda + r] : T(0);
  }

  // the candidates of column 0, as loaded
  {
    K bk = 0;
    int bi = 0x7fffffff;
#pragma unroll
    for (int q = 0; q < RPT; ++q)
      if (pos[q] < m) {
        const K key = pivot_key<T>(v[q][0], pos[q] == 0);
        if (key > bk || (key == bk && pos[q] < bi)) { bk = key; bi = pos[q]; }
      }
    K ck;
    int ci;
    cluster_panel_cta_candidate<T, NB>(sh, bk, bi, ck, ci);
    const bool ow = ci != 0x7fffffff && sh.widx[warp] == ci;
    if (ow) {
#pragma unroll
      for (int q = 0; q < RPT; ++q)
        if (pos[q] == ci) {
#pragma unroll
          for (int c = 0; c < NB; ++c) sh.outrow[c] = v[q][c];
        }
      __syncwarp();
    }
    cluster_arrive(cluster_panel_push<T, NB>(sh, 0, ck, ci, ow, C, rank));
    cluster_wait();
  }

  int sl = 0;
#pragma unroll 1
  for (int j = 0; j < nbc; ++j) {
    // 1. every warp picks the same winner from the local copies
    K wk = lane < C ? sh.ckey[sl][lane] : (K)0;
    int wi = lane < C ? sh.cidx[sl][lane] : 0x7fffffff;
    warp_keymax(wk, wi);
    const int p = wi;
    const int cw = __ffs(__ballot_sync(0xffffffffu, lane < C && sh.cidx[sl][lane] == p)) - 1;
    const T* u = sh.crows[sl][cw];
    const T piv = u[0];
    const bool nz = (piv != T(0));   // biggest_in_corner != 0 (NaN counts as nonzero)
    if (tid == 0) sh.spiv[j] = p;
    if (keeper) {
      tr[j] = k0 + p;
      if (nz && p != j) ++swaps;
      if (!nz && first_zero < 0) first_zero = k0 + j;
    }
    T l[RPT];
    bool live[RPT];
#pragma unroll
    for (int q = 0; q < RPT; ++q) {
      const int r = pos[q];
      const int slot = tid + q * kClusterPanelThreads;
      if (r == p) {
        // the pivot row: its values are row j of U (the row it stored)
#pragma unroll
        for (int c = 0; c < NB; ++c)
          if (j + c < nbc) fin[(j + c) * S + slot] = v[q][c];
        pos[q] = j;
      } else if (r == j && nz) {
        pos[q] = p;                  // the row at position j takes the pivot row's place
      }
      live[q] = pos[q] < m && pos[q] > j;
      l[q] = T(0);
      if (live[q]) {
        T lq = v[q][0];
        if (nz) lq = lq / piv;
        l[q] = lq;
        fin[j * S + slot] = lq;
        v[q][1] = fma(-lq, u[1], v[q][1]);
      }
    }
    if (j + 1 == nbc) break;
    const int sn = sl == 2 ? 0 : sl + 1;
    // 2. the candidates of column j+1
    K bk = 0;
    int bi = 0x7fffffff;
#pragma unroll
    for (int q = 0; q < RPT; ++q)
      if (live[q]) {
        const K key = pivot_key<T>(v[q][1], pos[q] == j + 1);
        if (key > bk || (key == bk && pos[q] < bi)) { bk = key; bi = pos[q]; }
      }
    K ck;
    int ci;
    cluster_panel_cta_candidate<T, NB>(sh, bk, bi, ck, ci);
    const bool ow = ci != 0x7fffffff && sh.widx[warp] == ci;
    bool done[RPT];
#pragma unroll
    for (int q = 0; q < RPT; ++q) done[q] = false;
    if (ow) {
#pragma unroll
      for (int q = 0; q < RPT; ++q)
        if (pos[q] == ci) {
          cluster_panel_shift_update<T, NB>(v[q], l[q], u);
#pragma unroll
          for (int c = 0; c < NB; ++c) sh.outrow[c] = v[q][c];
          done[q] = true;
        }
      __syncwarp();
    }
    cluster_arrive(cluster_panel_push<T, NB>(sh, sn, ck, ci, ow, C, rank));
    // 3. the rank-1 update of the other columns while the barrier completes
#pragma unroll
    for (int q = 0; q < RPT; ++q)
      if (live[q] && !done[q]) cluster_panel_shift_update<T, NB>(v[q], l[q], u);
    cluster_wait();
    sl = sn;
  }
  if (keeper) {
    if (swaps) st->nb_transpositions += swaps;
    if (first_zero >= 0 && st->info < 0) st->info = first_zero;
  }

  __syncthreads();
#pragma unroll
  for (int q = 0; q < RPT; ++q) {
    const int r = pos[q];
    if (r < m) {
      const int slot = tid + q * kClusterPanelThreads;
      for (int c = 0; c < nbc; ++c) a[(int64_t)c * lda + r] = fin[c * S + slot];
    }
  }
  // the fused TRSM below reads L11, whose rows other CTAs may have written;
  // without it, no CTA touches another's shared memory after the last barrier
  if (trsm_cols > 0) cluster.sync();

  if (rank == 0 && (map || trsm_cols > 0)) cluster_panel_tail<T, NB>(sh, a, lda, m, nbc, k0, map, trsm_cols);
}

// ---------------------------------------------------------------- tournament pivoting
// Panel LU with tournament pivoting (CALU: Grigori, Demmel, Xiang, "CALU: a
// communication optimal LU factorization algorithm", SIAM J. Matrix Anal.
// Appl. 32(4), 2011), for the mixed-precision path, whose refinement (and FP64
// fallback) needs a stable factorization but not the reference's pivot order.
// The panel's pivots come from a reduction of candidate rows instead of one
// cluster-wide argmax per column:
//   1. every CTA runs partial pivoting on its own rows (one row per thread,
//      CTA barriers only) to pick NB candidate rows, and stores their original
//      values into CTA 0's shared memory;
//   2. cluster barrier; CTA 0 runs partial pivoting on the C NB stacked
//      candidates: their order is the panel's pivot order and the pivot rows,
//      eliminated, are U11; one warp turns the order into transpositions;
//   3. cluster barrier; every CTA copies U11, the order and the transpositions,
//      and each thread forms its row of L (row r: the solution of
//      l U11 = a_r over the columns before its pivot step, or all columns) from
//      the row's original values, writing each entry once at the row's final
//      position.
// Two cluster barriers per panel instead of NB.  A zero pivot is reported as
// the first zero pivot (the caller then falls back).  The row map and the
// fused U12 solve are the partial-pivoting kernel's (cluster_panel_tail).
template <typename T, int NB>
struct TournamentShared {
  typedef typename PivotKey<T>::type K;
  static constexpr int NW = kClusterPanelThreads / 32;
  __align__(16) T wrow[2][NW][NB];    // each warp's best row, by step parity
  K wkey[2][NW];
  int widx[2][NW];
  int S[NB];                          // pivot order (panel-relative rows), CTA 0's result
  int spiv[NB];                       // transpositions: step j swaps positions j and spiv[j]
  __align__(16) T u11[NB][2 * NB];    // U11, row i = pivot i after elimination (columns i..NB-1; zero elsewhere)
  T rdiag[NB];                        // 1 / U11(i, i), 0 for a zero pivot
  int first_zero;                     // first step with a zero pivot, or -1
  int tgt[2 * NB], src[2 * NB];
  T l11[NB][NB + 1];
};

template <typename T, int NB>
constexpr size_t tournament_dyn_smem()
{
  return (sizeof(T) * NB + sizeof(int)) * (size_t)kMaxPanelCluster * NB;   // stacked candidates + their rows
}

// Partial pivoting over the CTA's rows, one row per thread (v: the row's
// columns, rotated so that the current column is v[0]; id: its panel row,
// valid: it takes part).  Returns the step at which this thread's row was
// chosen, or -1.  record: CTA 0's final round; it also writes sh.S, sh.u11,
// sh.rdiag and sh.first_zero.  One CTA barrier per step (the staging rows are
// double-buffered by step parity).
template <typename T, int NB>
__device__ int tournament_gepp(TournamentShared<T, NB>& sh, T (&v)[NB], int id, bool valid, bool record)
{
  typedef typename PivotKey<T>::type K;
  constexpr int NW = kClusterPanelThreads / 32;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  int chosen = -1;
#pragma unroll 1
  for (int j = 0; j < NB; ++j) {
    const int b = j & 1;
    K bk = valid ? pivot_key<T>(v[0], false) : (K)0;
    int bi = valid ? id : 0x7fffffff;
    warp_keymax(bk, bi);
    if (valid && id == bi) {                       // this warp's best row, staged for the CTA
#pragma unroll
      for (int c = 0; c < NB; ++c) sh.wrow[b][warp][c] = v[c];
      sh.wkey[b][warp] = bk;
      sh.widx[b][warp] = bi;
    } else if (lane == 0 && bi == 0x7fffffff) {
      sh.wkey[b][warp] = (K)0;
      sh.widx[b][warp] = 0x7fffffff;
    }
    __syncthreads();
    K ck = lane < NW ? sh.wkey[b][lane] : (K)0;
    int ci = lane < NW ? sh.widx[b][lane] : 0x7fffffff;
    warp_keymax(ck, ci);
    if (ci == 0x7fffffff) {                        // no rows left (fewer than NB valid rows)
      if (record && tid == 0) {
        sh.S[j] = -1;
        sh.rdiag[j] = T(0);
        if (sh.first_zero < 0) sh.first_zero = j;
      }
      if (record && tid < 2 * NB) sh.u11[j][tid] = T(0);
      continue;
    }
    const int cw = __ffs(__ballot_sync(0xffffffffu, lane < NW && sh.widx[b][lane] == ci)) - 1;
    const T* u = sh.wrow[b][cw];
    const T piv = u[0];
    const bool nz = piv != T(0);
    if (record && tid == 0) {
      sh.S[j] = ci;
      sh.rdiag[j] = nz ? T(1) / piv : T(0);
      if (!nz && sh.first_zero < 0) sh.first_zero = j;
    }
    if (record && tid < 2 * NB) sh.u11[j][tid] = (tid >= j && tid < NB) ? u[tid - j] : T(0);
    if (valid && id == ci) {
      valid = false;
      chosen = j;
    }
    if (valid) {                                   // eliminate column j, shift the row left by one slot
      const T l = nz ? v[0] * (T(1) / piv) : v[0];
#pragma unroll
      for (int c = 0; c < NB - 1; ++c) v[c] = fma(-l, u[c + 1], v[c + 1]);
      v[NB - 1] = T(0);
    }
  }
  return chosen;
}

// a: the panel (m rows, NB columns) at row and column k0 of its matrix, on a
// cluster of C CTAs with C * kClusterPanelThreads >= m; tr, st, map and
// trsm_cols as for panel_lu_cluster_kernel.  Dynamic shared memory:
// tournament_dyn_smem<T, NB>() (CTA 0's stacked candidates).
template <typename T, int NB>
__global__ void __launch_bounds__(kClusterPanelThreads)
panel_lu_tournament_kernel(T* __restrict__ a, int64_t lda, int m, int k0, int* __restrict__ tr, DeviceStatus* st,
                           int* __restrict__ map, int trsm_cols)
{
  static_assert(NB == 32, "one lane per panel column");
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  const int C = (int)cluster.num_blocks();
  const int rank = (int)cluster.block_rank();
  __shared__ TournamentShared<T, NB> sh;
  extern __shared__ __align__(16) unsigned char tournament_dyn[];
  T* cand = reinterpret_cast<T*>(tournament_dyn);                                   // [C NB][NB] in CTA 0
  int* cand_row = reinterpret_cast<int*>(tournament_dyn + sizeof(T) * kMaxPanelCluster * NB * NB);   // [C NB]
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int r = rank * kClusterPanelThreads + tid;      // this thread's panel row
  const bool mine = r < m;
  if (tid == 0) sh.first_zero = -1;

  // 0. the row; its original values stay in o for the final solve
  T o[NB], v[NB];
#pragma unroll
  for (int c = 0; c < NB; ++c) {
    o[c] = mine ? a[(int64_t)c * lda + r] : T(0);
    v[c] = o[c];
  }
  __syncthreads();

  // 1. this CTA's candidates, original values, into CTA 0 in the order chosen;
  //    the steps after the CTA's rows ran out leave their slots empty
  const int step = tournament_gepp<T, NB>(sh, v, r, mine, false);
  const int nvalid = min(NB, max(0, m - rank * kClusterPanelThreads));
  bool wrote = false;
  {
    T* cand0 = cluster.map_shared_rank(cand, 0);
    int* row0 = cluster.map_shared_rank(cand_row, 0);
    if (step >= 0) {
      const int slot = rank * NB + step;
#pragma unroll
      for (int c = 0; c < NB; ++c) cand0[slot * NB + c] = o[c];
      row0[slot] = r;
      wrote = true;
    }
    if (tid >= nvalid && tid < NB) {
      row0[rank * NB + tid] = -1;
      wrote = true;
    }
  }
  cluster_arrive(__any_sync(0xffffffffu, wrote));
  cluster_wait();

  // 2. CTA 0: partial pivoting on the stacked candidates gives the order and
  //    U11; one warp turns the order into transpositions
  if (rank == 0) {
    const bool cv = tid < C * NB && cand_row[tid] >= 0;
    T w[NB];
#pragma unroll
    for (int c = 0; c < NB; ++c) w[c] = cv ? cand[tid * NB + c] : T(0);
    tournament_gepp<T, NB>(sh, w, cv ? cand_row[tid] : 0x7fffffff, cv, true);
    __syncthreads();
    if (warp == 0) {
      // lane k keeps (the row that was at position k before step k, where it went)
      int myR = -1, myP = -1;
      for (int j = 0; j < NB; ++j) {
        const int sj = sh.S[j];
        int p = j;
        if (sj >= 0) {
          const unsigned mk = __ballot_sync(0xffffffffu, lane < j && myR == sj);
          const int kk = mk ? 31 - __clz(mk) : 0;
          const int pk = __shfl_sync(0xffffffffu, myP, kk);
          p = mk ? pk : sj;
        }
        const unsigned mp = __ballot_sync(0xffffffffu, lane < j && myP == j);
        const int kr = mp ? 31 - __clz(mp) : 0;
        const int rk = __shfl_sync(0xffffffffu, myR, kr);
        const int R = mp ? rk : j;
        if (lane == j) {
          myR = R;
          myP = p;
        }
        if (lane == 0) sh.spiv[j] = p;
      }
    }
    __syncthreads();
  }
  cluster_arrive(rank == 0);
  cluster_wait();

  // 3. every CTA: U11, order and transpositions from CTA 0, then the rows of L
  if (rank != 0) {
    const TournamentShared<T, NB>* s0 = cluster.map_shared_rank(&sh, 0);
    for (int e = tid; e < NB * 2 * NB; e += kClusterPanelThreads) (&sh.u11[0][0])[e] = (&s0->u11[0][0])[e];
    if (tid < NB) {
      sh.S[tid] = s0->S[tid];
      sh.spiv[tid] = s0->spiv[tid];
      sh.rdiag[tid] = s0->rdiag[tid];
    }
    __syncthreads();
  }
  cluster_arrive(false);                    // done with CTA 0's shared memory (waited for below)
  if (mine) {
    int ps = -1;                            // the step at which this row is the pivot
    for (int j = 0; j < NB; ++j)
      if (sh.S[j] == r) ps = j;
    int pos = r;
    for (int j = 0; j < NB; ++j) {
      const int p = sh.spiv[j];
      if (pos == j) pos = p;
      else if (pos == p) pos = j;
    }
    // t[c] = column j + c of a_r - l U11 so far (rotated like the factorization)
#pragma unroll 1
    for (int j = 0; j < NB; ++j) {
      if (j == ps) {
        for (int c = j; c < NB; ++c) a[(int64_t)c * lda + pos] = sh.u11[j][c];
        break;
      }
      const T rd = sh.rdiag[j];
      const T l = rd != T(0) ? o[0] * rd : o[0];
      a[(int64_t)j * lda + pos] = l;
#pragma unroll
      for (int c = 0; c < NB - 1; ++c) o[c] = fma(-l, sh.u11[j][j + 1 + c], o[c + 1]);
      o[NB - 1] = T(0);
    }
  }
  cluster_wait();

  if (rank == 0) {
    if (tid < NB) tr[tid] = k0 + sh.spiv[tid];
    if (tid == 0) {
      int swaps = 0;
      for (int j = 0; j < NB; ++j) swaps += sh.spiv[j] != j;
      if (swaps) st->nb_transpositions += swaps;
      if (sh.first_zero >= 0 && st->info < 0) st->info = k0 + sh.first_zero;
    }
  }
  if (trsm_cols > 0) {                      // the panel's rows, written by every CTA, before CTA 0 reads L11
    cluster_arrive(true);
    cluster_wait();
  }
  if (rank == 0 && (map || trsm_cols > 0)) cluster_panel_tail<T, NB>(sh, a, lda, m, NB, k0, map, trsm_cols);
}

}  // namespace gbs
