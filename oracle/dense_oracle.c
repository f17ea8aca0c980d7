/*
 * Test infrastructure: the CPU oracle (results to compare against) for the
 * dense factor-and-solve path.  Not part of the product; only tests/, the smoke check and the
 * benchmark's CPU-baseline leg load it.  See dense_oracle_impl.h for the
 * reference functions each routine restates.
 *
 * Also holds the seeded, byte-stable input generators shared by the tests and
 * the fixture script: a counter-based splitmix64 hash gives each (seed, index)
 * 64 random bits, so entry (i,j) does not depend on how the matrix is split
 * over threads or machines, and the values involve integer arithmetic plus one
 * exact power-of-two scaling only (no libm), so x86 and Arm hosts produce
 * identical bytes.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define T double
#define SFX(name) name##_d
#define SQRT(x) sqrt(x)
#include "dense_oracle_impl.h"
#undef T
#undef SFX
#undef SQRT
#undef AT

#define T float
#define SFX(name) name##_s
#define SQRT(x) sqrtf(x)
#include "dense_oracle_impl.h"
#undef T
#undef SFX
#undef SQRT

static inline uint64_t mix64(uint64_t z)
{
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

static inline uint64_t hash2(uint64_t seed, uint64_t idx)
{
  return mix64(seed * 0x9E3779B97F4A7C15ULL + (idx + 1) * 0xD1B54A32D192ED03ULL);
}

/* Irwin-Hall(12) approximation of N(0,1): the sum of twelve 16-bit uniforms,
 * centred, divided by 65536 -- an exact value in both float and double. */
double oracle_gauss(uint64_t seed, uint64_t idx)
{
  uint64_t h0 = hash2(seed, 3 * idx), h1 = hash2(seed, 3 * idx + 1), h2 = hash2(seed, 3 * idx + 2);
  int64_t s = 0;
  for (int k = 0; k < 4; ++k) {
    s += (int64_t)((h0 >> (16 * k)) & 0xFFFF);
    s += (int64_t)((h1 >> (16 * k)) & 0xFFFF);
    s += (int64_t)((h2 >> (16 * k)) & 0xFFFF);
  }
  return (double)(2 * s - 786420) / 131072.0;
}

/* uniform in [-1, 1) with 2^-31 resolution (the reference tests use
 * MatrixXd::Random, uniform in [-1, 1]) */
double oracle_uniform(uint64_t seed, uint64_t idx)
{
  uint64_t h = hash2(seed, idx);
  return (double)((int64_t)(h >> 32) - 2147483648LL) / 2147483648.0;
}

void oracle_fill_gauss(uint64_t seed, long m, long n, double *a, long lda)
{
#pragma omp parallel for schedule(static) if ((double)m * n > 1e5)
  for (long j = 0; j < n; ++j)
    for (long i = 0; i < m; ++i) a[(size_t)j * lda + i] = oracle_gauss(seed, (uint64_t)j * (uint64_t)m + (uint64_t)i);
}

void oracle_fill_uniform(uint64_t seed, long m, long n, double *a, long lda)
{
#pragma omp parallel for schedule(static) if ((double)m * n > 1e5)
  for (long j = 0; j < n; ++j)
    for (long i = 0; i < m; ++i) a[(size_t)j * lda + i] = oracle_uniform(seed, (uint64_t)j * (uint64_t)m + (uint64_t)i);
}

/* A = G G^T / scale + shift I, exactly symmetric (lower computed, mirrored). */
void oracle_make_spd(uint64_t seed, long n, double scale, double shift, double *a, long lda)
{
  double *g = (double *)malloc(sizeof(double) * (size_t)n * (size_t)n);
  oracle_fill_gauss(seed, n, n, g, n);
#pragma omp parallel for schedule(dynamic, 8)
  for (long j = 0; j < n; ++j) {
    for (long i = j; i < n; ++i) {
      double s = 0;
      for (long k = 0; k < n; ++k) s += g[(size_t)k * n + i] * g[(size_t)k * n + j];
      s = s / scale + (i == j ? shift : 0.0);
      a[(size_t)j * lda + i] = s;
      a[(size_t)i * lda + j] = s;
    }
  }
  free(g);
}

/* normwise backward error max_r ||b - A x||_inf / (||A||_inf ||x||_inf + ||b||_inf),
 * computed in long double accumulation. */
double oracle_backward_error(long n, const double *a, long lda, long nrhs, const double *x, long ldx,
                             const double *b, long ldb)
{
  double anorm = 0;
  for (long i = 0; i < n; ++i) {
    double s = 0;
    for (long j = 0; j < n; ++j) s += fabs(a[(size_t)j * lda + i]);
    if (s > anorm) anorm = s;
  }
  double worst = 0;
  for (long r = 0; r < nrhs; ++r) {
    const double *xr = x + (size_t)r * ldx, *br = b + (size_t)r * ldb;
    double rn = 0, xn = 0, bn = 0;
    for (long i = 0; i < n; ++i) {
      long double s = br[i];
      for (long j = 0; j < n; ++j) s -= (long double)a[(size_t)j * lda + i] * xr[j];
      if (fabsl(s) > rn) rn = (double)fabsl(s);
      if (fabs(xr[i]) > xn) xn = fabs(xr[i]);
      if (fabs(br[i]) > bn) bn = fabs(br[i]);
    }
    double den = anorm * xn + bn;
    double e = den > 0 ? rn / den : rn;
    if (e > worst) worst = e;
  }
  return worst;
}

int oracle_num_threads(void)
{
#ifdef _OPENMP
  extern int omp_get_max_threads(void);
  return omp_get_max_threads();
#else
  return 1;
#endif
}
