/* Test double of the plug-in level of libgb300solve (the four functions
 * include/eigen_gb300/GB300Support calls), for CPU-only tests of the header's
 * glue: it counts calls and forwards to the C oracle's restatement of the
 * reference algorithms.  Test infrastructure only. */
#include <stdint.h>

long oracle_llt_blocked_d(long n, double *a, long lda);
long oracle_llt_blocked_upper_d(long n, double *a, long lda);
long oracle_llt_blocked_s(long n, float *a, long lda);
long oracle_llt_blocked_upper_s(long n, float *a, long lda);
long oracle_lu_blocked_d(long rows, long cols, double *lu, long ld, int *tr, int *nb_tr, long maxBlockSize);
long oracle_lu_blocked_s(long rows, long cols, float *lu, long ld, int *tr, int *nb_tr, long maxBlockSize);

int gbs_mock_calls = 0;

int64_t gbs_llt_blocked_d(int64_t n, double *a, int64_t lda, int upper)
{
  ++gbs_mock_calls;
  return upper ? oracle_llt_blocked_upper_d(n, a, lda) : oracle_llt_blocked_d(n, a, lda);
}
int64_t gbs_llt_blocked_s(int64_t n, float *a, int64_t lda, int upper)
{
  ++gbs_mock_calls;
  return upper ? oracle_llt_blocked_upper_s(n, a, lda) : oracle_llt_blocked_s(n, a, lda);
}
int64_t gbs_partial_lu_blocked_d(int64_t r, int64_t c, double *a, int64_t lda, int *tr, int *nbt)
{
  ++gbs_mock_calls;
  return oracle_lu_blocked_d(r, c, a, lda, tr, nbt, 256);
}
int64_t gbs_partial_lu_blocked_s(int64_t r, int64_t c, float *a, int64_t lda, int *tr, int *nbt)
{
  ++gbs_mock_calls;
  return oracle_lu_blocked_s(r, c, a, lda, tr, nbt, 256);
}
