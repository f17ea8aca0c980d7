/*
 * Test infrastructure: the CPU oracle for the dense factor-and-solve path.
 * Only the tests, the smoke check and the CPU-baseline leg of the benchmark use
 * this code, to check results or time the baseline.  The product (libgb300solve)
 * never links it.
 *
 * This file is included twice by dense_oracle.c, once with T=double and once
 * with T=float; SFX(name) appends the type suffix (_d / _s) and SQRT is the
 * correctly rounded square root of that type.
 *
 * It restates, in plain C and column-major storage, the algorithms of the
 * reference (Eigen 3.3.90):
 *   llt_unblocked   Eigen/src/Cholesky/LLT.h:305-328
 *   llt_blocked     Eigen/src/Cholesky/LLT.h:331-360 (bs = clamp((n/8)/16*16, 8, 128))
 *   lu_unblocked    Eigen/src/LU/PartialPivLU.h:365-409
 *   lu_blocked      Eigen/src/LU/PartialPivLU.h:426-496 (outer bs <= 256, inner 16)
 *   pivot rule      Eigen/src/Core/Visitor.h:173-186 (strict '>' : first max wins)
 *   l1 norms        LLT.h:434-445, PartialPivLU.h:522
 *   solves          LLT.h:477-505, PartialPivLU.h:224-271
 *   rcond           Eigen/src/Core/ConditionEstimator.h:56-169
 *   permutation     Eigen/src/Core/PermutationMatrix.h:82-88 (transpositions right to left)
 * The same blocking is kept so the operation order (and therefore the pivot
 * sequence) follows the reference; rounding inside the inner products differs
 * (summation order, FMA contraction), as it already does between two builds of
 * the reference itself.
 */

#define AT(a, lda, i, j) (a)[(size_t)(j) * (size_t)(lda) + (size_t)(i)]

/* ---------------------------------------------------------------- GEMM
 * C(m x n) -= A(m x k) * B(k x n), all column-major.  This is the trailing
 * update of PartialPivLU.h:492 (general_matrix_matrix_product, OpenMP over
 * column blocks as Parallelizer.h:86-157 does).  4-column register blocking,
 * k-blocks of 256 so the A block stays in L2.                              */
static void SFX(gemm_sub)(long m, long n, long k, const T *A, long lda,
                          const T *B, long ldb, T *C, long ldc)
{
  if (m <= 0 || n <= 0 || k <= 0) return;
  const long KB = 256, MB = 256;
  long njb = (n + 3) / 4;
#pragma omp parallel for schedule(dynamic, 4) if ((double)m * n * k > 2.0e6)
  for (long jb = 0; jb < njb; ++jb) {
    long j0 = jb * 4;
    long nj = n - j0 < 4 ? n - j0 : 4;
    for (long k0 = 0; k0 < k; k0 += KB) {
      long kk = k - k0 < KB ? k - k0 : KB;
      for (long i0 = 0; i0 < m; i0 += MB) {
        long mm = m - i0 < MB ? m - i0 : MB;
        if (nj == 4) {
          T *c0 = &AT(C, ldc, i0, j0 + 0), *c1 = &AT(C, ldc, i0, j0 + 1);
          T *c2 = &AT(C, ldc, i0, j0 + 2), *c3 = &AT(C, ldc, i0, j0 + 3);
          for (long p = k0; p < k0 + kk; ++p) {
            const T *a = &AT(A, lda, i0, p);
            T b0 = AT(B, ldb, p, j0 + 0), b1 = AT(B, ldb, p, j0 + 1);
            T b2 = AT(B, ldb, p, j0 + 2), b3 = AT(B, ldb, p, j0 + 3);
            for (long i = 0; i < mm; ++i) {
              T av = a[i];
              c0[i] -= av * b0; c1[i] -= av * b1;
              c2[i] -= av * b2; c3[i] -= av * b3;
            }
          }
        } else {
          for (long j = j0; j < j0 + nj; ++j) {
            T *c = &AT(C, ldc, i0, j);
            for (long p = k0; p < k0 + kk; ++p) {
              const T *a = &AT(A, lda, i0, p);
              T b = AT(B, ldb, p, j);
              for (long i = 0; i < mm; ++i) c[i] -= a[i] * b;
            }
          }
        }
      }
    }
  }
}

/* Lower triangle only: C(lower, n x n) -= A(n x k) * A^T.  SYRK of
 * LLT.h:357 (selfadjointView<Lower>().rankUpdate(A21,-1)); the strictly upper
 * part of C is never written (the reference leaves it untouched).  Column
 * blocks are independent, so they are spread over OpenMP threads. */
static void SFX(syrk_lower_sub)(long n, long k, const T *A, long lda, T *C, long ldc)
{
  if (n <= 0 || k <= 0) return;
  const long NB = 16;
  long nb = (n + NB - 1) / NB;
#pragma omp parallel for schedule(dynamic, 1) if ((double)n * n * k > 4.0e6)
  for (long b = 0; b < nb; ++b) {
    long j0 = b * NB;
    long nj = n - j0 < NB ? n - j0 : NB;
    for (long j = j0; j < j0 + nj; ++j) {
      T *c = &AT(C, ldc, 0, j);
      for (long p = 0; p < k; ++p) {
        T bv = AT(A, lda, j, p);
        const T *a = &AT(A, lda, 0, p);
        for (long i = j; i < n; ++i) c[i] -= a[i] * bv;
      }
    }
  }
}

/* X(m x bs) <- X * L^{-T}, L lower bs x bs (LLT.h:356, TRSM OnTheRight). */
static void SFX(trsm_right_lower_trans)(long m, long bs, const T *L, long ldl, T *X, long ldx)
{
  for (long j = 0; j < bs; ++j) {
    T *xj = &AT(X, ldx, 0, j);
    for (long l = 0; l < j; ++l) {
      T f = AT(L, ldl, j, l);
      const T *xl = &AT(X, ldx, 0, l);
      for (long i = 0; i < m; ++i) xj[i] -= xl[i] * f;
    }
    T d = AT(L, ldl, j, j);
    for (long i = 0; i < m; ++i) xj[i] /= d;
  }
}

/* B(bs x n) <- L^{-1} B, L unit lower bs x bs (PartialPivLU.h:490). */
static void SFX(trsm_left_unit_lower)(long bs, long n, const T *L, long ldl, T *B, long ldb)
{
#pragma omp parallel for schedule(static) if ((double)bs * bs * n > 4.0e6)
  for (long j = 0; j < n; ++j) {
    T *b = &AT(B, ldb, 0, j);
    for (long p = 0; p < bs; ++p) {
      T bp = b[p];
      for (long i = p + 1; i < bs; ++i) b[i] -= AT(L, ldl, i, p) * bp;
    }
  }
}

/* ---------------------------------------------------------------- LLT */
/* LLT.h:305-328.  Returns -1, or the first column whose pivot x <= 0. */
long SFX(oracle_llt_unblocked)(long n, T *a, long lda)
{
  for (long k = 0; k < n; ++k) {
    long rs = n - k - 1;
    T x = AT(a, lda, k, k);
    if (k > 0) {
      T s = 0;
      for (long j = 0; j < k; ++j) s += AT(a, lda, k, j) * AT(a, lda, k, j);
      x -= s;
    }
    if (x <= (T)0) return k;
    x = SQRT(x);
    AT(a, lda, k, k) = x;
    if (k > 0 && rs > 0) {
      for (long j = 0; j < k; ++j) {
        T f = AT(a, lda, k, j);
        for (long i = k + 1; i < n; ++i) AT(a, lda, i, k) -= AT(a, lda, i, j) * f;
      }
    }
    if (rs > 0)
      for (long i = k + 1; i < n; ++i) AT(a, lda, i, k) /= x;
  }
  return -1;
}

/* LLT.h:331-360. */
long SFX(oracle_llt_blocked)(long n, T *a, long lda)
{
  if (n < 32) return SFX(oracle_llt_unblocked)(n, a, lda);
  long blockSize = n / 8;
  blockSize = (blockSize / 16) * 16;
  if (blockSize < 8) blockSize = 8;
  if (blockSize > 128) blockSize = 128;
  for (long k = 0; k < n; k += blockSize) {
    long bs = blockSize < n - k ? blockSize : n - k;
    long rs = n - k - bs;
    long ret = SFX(oracle_llt_unblocked)(bs, &AT(a, lda, k, k), lda);
    if (ret >= 0) return k + ret;
    if (rs > 0) {
      SFX(trsm_right_lower_trans)(rs, bs, &AT(a, lda, k, k), lda, &AT(a, lda, k + bs, k), lda);
      SFX(syrk_lower_sub)(rs, bs, &AT(a, lda, k + bs, k), lda, &AT(a, lda, k + bs, k + bs), lda);
    }
  }
  return -1;
}

/* Upper mode (LLT.h:362-383): the reference factors the transpose view with
 * the lower algorithm; the same arithmetic is done here on a transposed copy
 * of the upper triangle, written back transposed.  Strictly lower part is
 * left untouched. */
long SFX(oracle_llt_blocked_upper)(long n, T *a, long lda)
{
  T *t = (T *)malloc(sizeof(T) * (size_t)(n > 0 ? n : 1) * (size_t)(n > 0 ? n : 1));
  for (long j = 0; j < n; ++j)
    for (long i = 0; i < n; ++i) AT(t, n, i, j) = (i >= j) ? AT(a, lda, j, i) : (T)0;
  long ret = SFX(oracle_llt_blocked)(n, t, n);
  for (long j = 0; j < n; ++j)
    for (long i = j; i < n; ++i) AT(a, lda, j, i) = AT(t, n, i, j);
  free(t);
  return ret;
}

/* ‖A‖₁ of the symmetric matrix whose lower (uplo=0) or upper (uplo=1)
 * triangle is stored (LLT.h:434-445). */
double SFX(oracle_sym_l1_norm)(long n, const T *a, long lda, int uplo)
{
  T best = 0;
  for (long col = 0; col < n; ++col) {
    T s1 = 0, s2 = 0;
    if (uplo == 0) {
      for (long i = col; i < n; ++i) s1 += (T)fabs((double)AT(a, lda, i, col));
      for (long j = 0; j < col; ++j) s2 += (T)fabs((double)AT(a, lda, col, j));
    } else {
      for (long i = 0; i < col; ++i) s1 += (T)fabs((double)AT(a, lda, i, col));
      for (long j = col; j < n; ++j) s2 += (T)fabs((double)AT(a, lda, col, j));
    }
    T s = s1 + s2;
    if (s > best) best = s;
  }
  return (double)best;
}

/* x <- (L L^T)^{-1} x for nrhs columns (LLT.h:499-505); L in the lower
 * triangle of a (uplo=0) or U = L^T in the upper triangle (uplo=1). */
void SFX(oracle_llt_solve)(long n, const T *a, long lda, int uplo, long nrhs, T *b, long ldb)
{
  for (long r = 0; r < nrhs; ++r) {
    T *x = &AT(b, ldb, 0, r);
    /* forward: L y = b, L(i,j) = uplo ? a(j,i) : a(i,j) */
    for (long j = 0; j < n; ++j) {
      x[j] /= AT(a, lda, j, j);
      T xj = x[j];
      if (uplo == 0) for (long i = j + 1; i < n; ++i) x[i] -= AT(a, lda, i, j) * xj;
      else           for (long i = j + 1; i < n; ++i) x[i] -= AT(a, lda, j, i) * xj;
    }
    /* backward: L^T x = y */
    for (long i = n - 1; i >= 0; --i) {
      T s = x[i];
      if (uplo == 0) for (long k = i + 1; k < n; ++k) s -= AT(a, lda, k, i) * x[k];
      else           for (long k = i + 1; k < n; ++k) s -= AT(a, lda, i, k) * x[k];
      x[i] = s / AT(a, lda, i, i);
    }
  }
}

/* ---------------------------------------------------------------- LU */
static inline T SFX(absv)(T v) { return v < (T)0 ? -v : v; }

/* PartialPivLU.h:365-409 on a rows x cols block; pivots are 0-based and
 * relative to the block.  Returns the first exactly-zero pivot or -1. */
long SFX(oracle_lu_unblocked)(long rows, long cols, T *lu, long ld, int *tr, int *nb_tr)
{
  long size = rows < cols ? rows : cols;
  int nbt = 0;
  long first_zero = -1;
  for (long k = 0; k < size; ++k) {
    long rrows = rows - k - 1, rcols = cols - k - 1;
    /* maxCoeff(&idx) over |col k|, rows k.., strict '>' (Visitor.h:180) */
    long piv = k;
    T best = SFX(absv)(AT(lu, ld, k, k));
    for (long i = k + 1; i < rows; ++i) {
      T v = SFX(absv)(AT(lu, ld, i, k));
      if (v > best) { best = v; piv = i; }
    }
    tr[k] = (int)piv;
    if (best != (T)0) {
      if (piv != k) {
        for (long j = 0; j < cols; ++j) {
          T t = AT(lu, ld, k, j); AT(lu, ld, k, j) = AT(lu, ld, piv, j); AT(lu, ld, piv, j) = t;
        }
        ++nbt;
      }
      T d = AT(lu, ld, k, k);
      for (long i = k + 1; i < rows; ++i) AT(lu, ld, i, k) /= d;
    } else if (first_zero == -1) {
      first_zero = k;
    }
    if (k < rows - 1) {
      for (long j = k + 1; j < k + 1 + rcols; ++j) {
        T u = AT(lu, ld, k, j);
        for (long i = k + 1; i < k + 1 + rrows; ++i) AT(lu, ld, i, j) -= AT(lu, ld, i, k) * u;
      }
    }
  }
  *nb_tr = nbt;
  return first_zero;
}

static void SFX(swap_rows)(T *a, long ld, long ncols, long r1, long r2)
{
  if (r1 == r2) return;
  for (long j = 0; j < ncols; ++j) {
    T t = AT(a, ld, r1, j); AT(a, ld, r1, j) = AT(a, ld, r2, j); AT(a, ld, r2, j) = t;
  }
}

/* PartialPivLU.h:426-496, with the same recursive blocking. */
long SFX(oracle_lu_blocked)(long rows, long cols, T *lu, long ld, int *tr, int *nb_tr, long maxBlockSize)
{
  long size = rows < cols ? rows : cols;
  if (size <= 16) return SFX(oracle_lu_unblocked)(rows, cols, lu, ld, tr, nb_tr);
  long blockSize = size / 8;
  blockSize = (blockSize / 16) * 16;
  if (blockSize < 8) blockSize = 8;
  if (blockSize > maxBlockSize) blockSize = maxBlockSize;
  int nbt = 0;
  long first_zero = -1;
  for (long k = 0; k < size; k += blockSize) {
    long bs = size - k < blockSize ? size - k : blockSize;
    long trows = rows - k - bs;
    long tsize = size - k - bs;
    int nbt_panel = 0;
    long ret = SFX(oracle_lu_blocked)(trows + bs, bs, &AT(lu, ld, k, k), ld, tr + k, &nbt_panel, 16);
    if (ret >= 0 && first_zero == -1) first_zero = k + ret;
    nbt += nbt_panel;
    for (long i = k; i < k + bs; ++i) {
      tr[i] += (int)k;
      SFX(swap_rows)(lu, ld, k, i, tr[i]);                   /* A_0 */
    }
    if (trows) {
      for (long i = k; i < k + bs; ++i)
        SFX(swap_rows)(&AT(lu, ld, 0, k + bs), ld, tsize, i, tr[i]);  /* A_2 */
      SFX(trsm_left_unit_lower)(bs, tsize, &AT(lu, ld, k, k), ld, &AT(lu, ld, k, k + bs), ld);
      SFX(gemm_sub)(trows, tsize, bs, &AT(lu, ld, k + bs, k), ld, &AT(lu, ld, k, k + bs), ld,
                    &AT(lu, ld, k + bs, k + bs), ld);
    }
  }
  *nb_tr = nbt;
  return first_zero;
}

/* max column abs-sum (PartialPivLU.h:522) */
double SFX(oracle_l1_norm)(long m, long n, const T *a, long lda)
{
  T best = 0;
  for (long j = 0; j < n; ++j) {
    T s = 0;
    for (long i = 0; i < m; ++i) s += SFX(absv)(AT(a, lda, i, j));
    if (s > best) best = s;
  }
  return (double)best;
}

/* Transpositions -> permutation indices (PermutationMatrix.h:82-88). */
void SFX(oracle_perm_from_transpositions)(long n, const int *tr, int *perm)
{
  for (long i = 0; i < n; ++i) perm[i] = (int)i;
  for (long k = n - 1; k >= 0; --k) {
    int t = perm[k]; perm[k] = perm[tr[k]]; perm[tr[k]] = t;
  }
}

/* x = A^{-1} b with PA = LU (PartialPivLU.h:224-244): dst = P b (row
 * perm[i] of dst = row i of b), then unit-lower and upper substitution. */
void SFX(oracle_lu_solve)(long n, const T *lu, long ld, const int *tr, long nrhs, T *b, long ldb)
{
  int *perm = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
  T *tmp = (T *)malloc(sizeof(T) * (size_t)(n > 0 ? n : 1));
  SFX(oracle_perm_from_transpositions)(n, tr, perm);
  for (long r = 0; r < nrhs; ++r) {
    T *x = &AT(b, ldb, 0, r);
    for (long i = 0; i < n; ++i) tmp[perm[i]] = x[i];
    for (long i = 0; i < n; ++i) x[i] = tmp[i];
    for (long j = 0; j < n; ++j) {
      T xj = x[j];
      for (long i = j + 1; i < n; ++i) x[i] -= AT(lu, ld, i, j) * xj;
    }
    for (long j = n - 1; j >= 0; --j) {
      x[j] /= AT(lu, ld, j, j);
      T xj = x[j];
      for (long i = 0; i < j; ++i) x[i] -= AT(lu, ld, i, j) * xj;
    }
  }
  free(tmp);
  free(perm);
}

/* x = A^{-T} b (PartialPivLU.h:246-271): U^T solve, unit L^T solve, then
 * dst = P^T dst (row i of dst = row perm[i]). */
void SFX(oracle_lu_solve_transposed)(long n, const T *lu, long ld, const int *tr, long nrhs, T *b, long ldb)
{
  int *perm = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
  T *tmp = (T *)malloc(sizeof(T) * (size_t)(n > 0 ? n : 1));
  SFX(oracle_perm_from_transpositions)(n, tr, perm);
  for (long r = 0; r < nrhs; ++r) {
    T *x = &AT(b, ldb, 0, r);
    for (long i = 0; i < n; ++i) {          /* U^T y = b, forward */
      T s = x[i];
      for (long k = 0; k < i; ++k) s -= AT(lu, ld, k, i) * x[k];
      x[i] = s / AT(lu, ld, i, i);
    }
    for (long i = n - 1; i >= 0; --i) {     /* L^T z = y, backward, unit */
      T s = x[i];
      for (long k = i + 1; k < n; ++k) s -= AT(lu, ld, k, i) * x[k];
      x[i] = s;
    }
    for (long i = 0; i < n; ++i) tmp[i] = x[perm[i]];
    for (long i = 0; i < n; ++i) x[i] = tmp[i];
  }
  free(tmp);
  free(perm);
}

/* ---------------------------------------------------------------- rcond
 * ConditionEstimator.h:56-142 (Hager / Higham 1-norm estimate of inv(A)) and
 * :157-169 (rcond_estimate_helper).  kind 3 = LDLT (a holds L and D, tr the
 * transpositions; the solve is self-adjoint).  kind 0 = LU (a holds LU, tr the
 * transpositions), kind 1 = LLT lower, kind 2 = LLT upper. */
void SFX(oracle_ldlt_solve)(long n, const T *a, long lda, const int *tr, long nrhs, T *b, long ldb);

static void SFX(dec_solve)(int kind, long n, const T *a, long lda, const int *tr, T *v, int adjoint)
{
  if (kind == 0) {
    if (adjoint) SFX(oracle_lu_solve_transposed)(n, a, lda, tr, 1, v, n);
    else         SFX(oracle_lu_solve)(n, a, lda, tr, 1, v, n);
  } else if (kind == 3) {
    SFX(oracle_ldlt_solve)(n, a, lda, tr, 1, v, n);   /* self-adjoint */
  } else {
    SFX(oracle_llt_solve)(n, a, lda, kind == 2, 1, v, n);
  }
}

static T SFX(l1v)(long n, const T *v)
{
  T s = 0;
  for (long i = 0; i < n; ++i) s += SFX(absv)(v[i]);
  return s;
}

double SFX(oracle_inv_l1_estimate)(int kind, long n, const T *a, long lda, const int *tr)
{
  if (n == 0) return 0.0;
  T *v = (T *)malloc(sizeof(T) * (size_t)n);
  T *sgn = (T *)malloc(sizeof(T) * (size_t)n);
  T *old_sgn = (T *)malloc(sizeof(T) * (size_t)n);
  for (long i = 0; i < n; ++i) v[i] = (T)1 / (T)n;
  SFX(dec_solve)(kind, n, a, lda, tr, v, 0);
  T lower_bound = SFX(l1v)(n, v);
  if (n == 1) { free(v); free(sgn); free(old_sgn); return (double)lower_bound; }
  T old_lower_bound = lower_bound;
  long vmax = -1, old_vmax = -1;
  for (int k = 0; k < 4; ++k) {
    for (long i = 0; i < n; ++i) sgn[i] = v[i] < (T)0 ? (T)-1 : (T)1;
    if (k > 0) {
      int same = 1;
      for (long i = 0; i < n; ++i) if (sgn[i] != old_sgn[i]) { same = 0; break; }
      if (same) break;
    }
    for (long i = 0; i < n; ++i) v[i] = sgn[i];
    SFX(dec_solve)(kind, n, a, lda, tr, v, 1);
    vmax = 0;
    T best = SFX(absv)(v[0]);
    for (long i = 1; i < n; ++i) { T t = SFX(absv)(v[i]); if (t > best) { best = t; vmax = i; } }
    if (vmax == old_vmax) break;
    for (long i = 0; i < n; ++i) v[i] = 0;
    v[vmax] = 1;
    SFX(dec_solve)(kind, n, a, lda, tr, v, 0);
    lower_bound = SFX(l1v)(n, v);
    if (lower_bound <= old_lower_bound) break;
    for (long i = 0; i < n; ++i) old_sgn[i] = sgn[i];
    old_vmax = vmax;
    old_lower_bound = lower_bound;
  }
  T alt = 1;
  for (long i = 0; i < n; ++i) {
    v[i] = alt * ((T)1 + ((T)i / (T)(n - 1)));
    alt = -alt;
  }
  SFX(dec_solve)(kind, n, a, lda, tr, v, 0);
  T alternate = ((T)2 * SFX(l1v)(n, v)) / ((T)3 * (T)n);
  free(v); free(sgn); free(old_sgn);
  return (double)(lower_bound > alternate ? lower_bound : alternate);
}

double SFX(oracle_rcond)(int kind, long n, const T *a, long lda, const int *tr, double matrix_norm)
{
  if (n == 0) return 1.0;
  if ((T)matrix_norm == (T)0) return 0.0;
  if (n == 1) return 1.0;
  T inv = (T)SFX(oracle_inv_l1_estimate)(kind, n, a, lda, tr);
  return inv == (T)0 ? 0.0 : (double)(((T)1 / inv) / (T)matrix_norm);
}

/* ---------------------------------------------------------------- LDLT
 * Eigen/src/Cholesky/LDLT.h:291-383, ldlt_inplace<Lower>::unblocked, on the
 * lower triangle.  Step k: the first maximum of |a_ii| over i = k..n-1 (the
 * diagonal beyond k is not updated yet, so the pivots follow the input's
 * diagonal; Visitor.h:173-186), the symmetric interchange written on the lower
 * triangle (:318-331), then the left-looking column (:339-344)
 *   t = D(0:k) A10^T,  a_kk -= A10 t,  A21 -= A20 t,
 * and A21 /= a_kk when |a_kk| > 0 (:354-357).  A zero (or NaN) pivot leaves
 * its column unscaled; the result is NumericalIssue when such a column is not
 * zero below the diagonal or a nonzero pivot follows a zero one (:356-360).
 * A zero first pivot (the whole diagonal zero) ends the factorization with
 * identity transpositions (:345-353).  sign uses the reference's SignMatrix
 * order: 0 PositiveSemiDef, 1 NegativeSemiDef, 2 ZeroSign, 3 Indefinite
 * (:362-369).  Returns 1 (Success) or 0 (NumericalIssue). */
int SFX(oracle_ldlt)(long n, T *a, long lda, int *tr, int *sign)
{
  *sign = 2;
  if (n <= 1) {
    if (n == 1) {
      tr[0] = 0;
      const T d = AT(a, lda, 0, 0);
      *sign = d > (T)0 ? 0 : d < (T)0 ? 1 : 2;
    }
    return 1;
  }
  T *temp = (T *)malloc(sizeof(T) * (size_t)n);
  int found_zero = 0, ret = 1;
  for (long k = 0; k < n; ++k) {
    long p = k;
    T best = SFX(absv)(AT(a, lda, k, k));
    for (long i = k + 1; i < n; ++i) {
      const T v = SFX(absv)(AT(a, lda, i, i));
      if (v > best) { best = v; p = i; }
    }
    tr[k] = (int)p;
    if (p != k) {
      const long s = n - p - 1;
      for (long j = 0; j < k; ++j) { T t = AT(a, lda, k, j); AT(a, lda, k, j) = AT(a, lda, p, j); AT(a, lda, p, j) = t; }
      for (long i = 0; i < s; ++i) {
        T t = AT(a, lda, p + 1 + i, k); AT(a, lda, p + 1 + i, k) = AT(a, lda, p + 1 + i, p); AT(a, lda, p + 1 + i, p) = t;
      }
      { T t = AT(a, lda, k, k); AT(a, lda, k, k) = AT(a, lda, p, p); AT(a, lda, p, p) = t; }
      for (long i = k + 1; i < p; ++i) { T t = AT(a, lda, i, k); AT(a, lda, i, k) = AT(a, lda, p, i); AT(a, lda, p, i) = t; }
    }
    const long rs = n - k - 1;
    if (k > 0) {
      for (long j = 0; j < k; ++j) temp[j] = AT(a, lda, j, j) * AT(a, lda, k, j);
      T dot = 0;
      for (long j = 0; j < k; ++j) dot += AT(a, lda, k, j) * temp[j];
      AT(a, lda, k, k) -= dot;
      for (long i = k + 1; i < n; ++i) {
        T acc = AT(a, lda, i, k);
        for (long j = 0; j < k; ++j) acc -= AT(a, lda, i, j) * temp[j];
        AT(a, lda, i, k) = acc;
      }
    }
    const T akk = AT(a, lda, k, k);
    const int valid = SFX(absv)(akk) > (T)0;
    if (k == 0 && !valid) {
      *sign = 2;
      for (long j = 0; j < n; ++j) {
        tr[j] = (int)j;
        for (long i = j + 1; i < n; ++i)
          if (!(AT(a, lda, i, j) == (T)0)) ret = 0;
      }
      free(temp);
      return ret;
    }
    if (rs > 0 && valid) {
      for (long i = k + 1; i < n; ++i) AT(a, lda, i, k) /= akk;
    } else if (rs > 0) {
      for (long i = k + 1; i < n; ++i)
        if (!(AT(a, lda, i, k) == (T)0)) ret = 0;
    }
    if (found_zero && valid) ret = 0;
    else if (!valid) found_zero = 1;
    if (*sign == 0) { if (akk < (T)0) *sign = 3; }
    else if (*sign == 1) { if (akk > (T)0) *sign = 3; }
    else if (*sign == 2) { if (akk > (T)0) *sign = 0; else if (akk < (T)0) *sign = 1; }
  }
  free(temp);
  return ret;
}

/* LDLT.h:540-577 (_solve_impl): b <- P b, L^-1, the pseudo-inverse of D
 * (entries with |d| <= 1/highest give zero), L^-T, P^T. */
void SFX(oracle_ldlt_solve)(long n, const T *a, long lda, const int *tr, long nrhs, T *b, long ldb)
{
  const T tol = (T)1 / (sizeof(T) == 8 ? (T)DBL_MAX : (T)FLT_MAX);
  for (long c = 0; c < nrhs; ++c) {
    T *x = b + (size_t)c * (size_t)ldb;
    for (long k = 0; k < n; ++k)
      if (tr[k] != k) { T t = x[k]; x[k] = x[tr[k]]; x[tr[k]] = t; }
    for (long j = 0; j < n; ++j)
      for (long i = j + 1; i < n; ++i) x[i] -= AT(a, lda, i, j) * x[j];
    for (long i = 0; i < n; ++i) {
      const T d = AT(a, lda, i, i);
      if (SFX(absv)(d) > tol) x[i] /= d;
      else x[i] = (T)0;
    }
    for (long j = n - 1; j >= 0; --j) {
      T s = x[j];
      for (long i = j + 1; i < n; ++i) s -= AT(a, lda, i, j) * x[i];
      x[j] = s;
    }
    for (long k = n - 1; k >= 0; --k)
      if (tr[k] != k) { T t = x[k]; x[k] = x[tr[k]]; x[tr[k]] = t; }
  }
}

/* ---------------------------------------------------------------- LLT rank update
 * Eigen/src/Cholesky/LLT.h:231-299 (llt_rank_update_lower) on the lower factor:
 * sigma > 0: Givens rotations, one per column (Jacobi.h:226-258 makeGivens of
 * (l_ii, -t_i), Jacobi.h:317-327 applied to the column and t); sigma <= 0:
 * the downdate, which stops at the first column whose new diagonal would not
 * be positive.  Returns that column or -1. */
long SFX(oracle_llt_rank_update)(long n, T *a, long lda, const T *vec, double sigma_d)
{
  const T sigma = (T)sigma_d;
  T *t = (T *)malloc(sizeof(T) * (size_t)(n > 0 ? n : 1));
  long ret = -1;
  if (sigma > (T)0) {
    const T ss = SQRT(sigma);
    for (long i = 0; i < n; ++i) t[i] = ss * vec[i];
    for (long i = 0; i < n; ++i) {
      const T p = AT(a, lda, i, i), q = -t[i];
      T c, s, r;
      if (q == (T)0) { c = p < (T)0 ? (T)-1 : (T)1; s = 0; r = SFX(absv)(p); }
      else if (p == (T)0) { c = 0; s = q < (T)0 ? (T)1 : (T)-1; r = SFX(absv)(q); }
      else if (SFX(absv)(p) > SFX(absv)(q)) {
        const T tt = q / p;
        T u = SQRT((T)1 + tt * tt);
        if (p < (T)0) u = -u;
        c = (T)1 / u; s = -tt * c; r = p * u;
      } else {
        const T tt = p / q;
        T u = SQRT((T)1 + tt * tt);
        if (q < (T)0) u = -u;
        s = -(T)1 / u; c = -tt * s; r = q * u;
      }
      AT(a, lda, i, i) = r;
      if (c == (T)1 && s == (T)0) continue;
      for (long k = i + 1; k < n; ++k) {
        const T xi = AT(a, lda, k, i), yi = t[k];
        AT(a, lda, k, i) = c * xi + s * yi;
        t[k] = -s * xi + c * yi;
      }
    }
  } else {
    for (long i = 0; i < n; ++i) t[i] = vec[i];
    T beta = 1;
    for (long j = 0; j < n; ++j) {
      const T ljj = AT(a, lda, j, j), dj = ljj * ljj, wj = t[j];
      const T swj2 = sigma * wj * wj, gamma = dj * beta + swj2;
      const T x = dj + swj2 / beta;
      if (x <= (T)0) { ret = j; break; }
      const T nljj = SQRT(x);
      AT(a, lda, j, j) = nljj;
      beta += swj2 / dj;
      const T f = wj / ljj;
      for (long k = j + 1; k < n; ++k) t[k] -= f * AT(a, lda, k, j);
      if (gamma != (T)0) {
        const T g1 = nljj / ljj, g2 = nljj * sigma * wj / gamma;
        for (long k = j + 1; k < n; ++k) AT(a, lda, k, j) = g1 * AT(a, lda, k, j) + g2 * t[k];
      }
    }
  }
  free(t);
  return ret;
}

/* ---------------------------------------------------------------- batched
 * The reference has no batch API; the CPU baseline is one decomposition per
 * matrix over an OpenMP parallel-for.  Matrices are packed back to back,
 * matrix b of size n_b at offset off[b] (elements), rhs at roff[b]. */
void SFX(oracle_batched_llt_solve)(long count, const int *ns, const long *off, T *a,
                                   const long *roff, T *rhs, int *info)
{
#pragma omp parallel for schedule(dynamic, 64)
  for (long b = 0; b < count; ++b) {
    long n = ns[b];
    long r = SFX(oracle_llt_blocked)(n, a + off[b], n);
    info[b] = (int)r;
    if (r < 0) SFX(oracle_llt_solve)(n, a + off[b], n, 0, 1, rhs + roff[b], n);
  }
}

void SFX(oracle_batched_lu_solve)(long count, const int *ns, const long *off, T *a,
                                  const long *roff, T *rhs, int *tr_out, int *info)
{
#pragma omp parallel for schedule(dynamic, 64)
  for (long b = 0; b < count; ++b) {
    long n = ns[b];
    int nbt = 0;
    long r = SFX(oracle_lu_blocked)(n, n, a + off[b], n, tr_out + roff[b], &nbt, 256);
    info[b] = (int)r;
    SFX(oracle_lu_solve)(n, a + off[b], n, tr_out + roff[b], 1, rhs + roff[b], n);
  }
}
