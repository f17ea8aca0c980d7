// Test infrastructure: a C wrapper over the reference (Eigen) itself, compiled
// from the read-only reference tree by oracle/build.py into oracle/_ref/.  It
// pins the plain-C oracle and generates the golden fixtures; nothing in the
// product links it.
//
// Each entry point runs the reference's public API exactly as a user would:
//   LLT<MatrixXd/MatrixXf, Lower|Upper>(A), .matrixLLT(), .info(), .solve(B), .rcond()
//   PartialPivLU<MatrixXd/MatrixXf>(A), .matrixLU(), .permutationP(), .solve(B),
//   .transpose().solve(B), .rcond(), .determinant()
//   LDLT<MatrixXd/MatrixXf, Lower|Upper>(A), .matrixLDLT(), .transpositionsP(),
//   .info(), .isPositive(), .isNegative(), .solve(B), .rcond()
#include <Eigen/Dense>
#include <cstring>

using namespace Eigen;

namespace {

template <typename S, int UpLo>
int llt_run(long n, const S* a, long lda, long nrhs, const S* b, long ldb, S* fact, S* x, double* rcond)
{
  typedef Matrix<S, Dynamic, Dynamic> M;
  Map<const M, 0, OuterStride<> > A(a, n, n, OuterStride<>(lda));
  LLT<M, UpLo> llt(A);
  Map<M>(fact, n, n) = llt.matrixLLT();
  int info = llt.info() == Success ? 0 : 1;
  if (info == 0) {
    if (nrhs > 0) {
      Map<const M, 0, OuterStride<> > B(b, n, nrhs, OuterStride<>(ldb));
      Map<M>(x, n, nrhs) = llt.solve(B);
    }
    if (rcond) *rcond = double(llt.rcond());
  }
  return info;
}

template <typename S>
int lu_run(long n, const S* a, long lda, long nrhs, const S* b, long ldb, S* fact, int* perm, S* x, S* xt,
           double* rcond, double* det)
{
  typedef Matrix<S, Dynamic, Dynamic> M;
  Map<const M, 0, OuterStride<> > A(a, n, n, OuterStride<>(lda));
  PartialPivLU<M> lu(A);
  Map<M>(fact, n, n) = lu.matrixLU();
  for (long i = 0; i < n; ++i) perm[i] = lu.permutationP().indices()(i);
  if (nrhs > 0) {
    Map<const M, 0, OuterStride<> > B(b, n, nrhs, OuterStride<>(ldb));
    Map<M>(x, n, nrhs) = lu.solve(B);
    if (xt) Map<M>(xt, n, nrhs) = lu.transpose().solve(B);
  }
  if (rcond) *rcond = double(lu.rcond());
  if (det) *det = double(lu.determinant());
  return 0;
}

// LDLT<Matrix, UpLo>(A): matrixLDLT(), transpositionsP().indices(), info(),
// isPositive() / isNegative() (flags[0], flags[1]), solve(B), rcond().
template <typename S, int UpLo>
int ldlt_run(long n, const S* a, long lda, long nrhs, const S* b, long ldb, S* fact, int* tr, S* x, double* rcond,
             int* flags)
{
  typedef Matrix<S, Dynamic, Dynamic> M;
  Map<const M, 0, OuterStride<> > A(a, n, n, OuterStride<>(lda));
  LDLT<M, UpLo> ldlt(A);
  Map<M>(fact, n, n) = ldlt.matrixLDLT();
  for (long i = 0; i < n; ++i) tr[i] = ldlt.transpositionsP().indices()(i);
  flags[0] = ldlt.isPositive() ? 1 : 0;
  flags[1] = ldlt.isNegative() ? 1 : 0;
  if (nrhs > 0) {
    Map<const M, 0, OuterStride<> > B(b, n, nrhs, OuterStride<>(ldb));
    Map<M>(x, n, nrhs) = ldlt.solve(B);
  }
  if (rcond) *rcond = double(ldlt.rcond());
  return ldlt.info() == Success ? 0 : 1;
}

// LLT<Matrix, UpLo>(A).rankUpdate(v, sigma): matrixLLT() and info() after the update.
template <typename S, int UpLo>
int llt_rank_update_run(long n, const S* a, long lda, const S* v, double sigma, S* fact)
{
  typedef Matrix<S, Dynamic, Dynamic> M;
  typedef Matrix<S, Dynamic, 1> V;
  Map<const M, 0, OuterStride<> > A(a, n, n, OuterStride<>(lda));
  LLT<M, UpLo> llt(A);
  if (llt.info() != Success) return 2;
  llt.rankUpdate(Map<const V>(v, n), S(sigma));
  Map<M>(fact, n, n) = llt.matrixLLT();
  return llt.info() == Success ? 0 : 1;
}

}  // namespace

extern "C" {

int ref_llt_rank_update_d(long n, const double* a, long lda, int upper, const double* v, double sigma, double* fact)
{
  return upper ? llt_rank_update_run<double, Upper>(n, a, lda, v, sigma, fact)
               : llt_rank_update_run<double, Lower>(n, a, lda, v, sigma, fact);
}

int ref_llt_rank_update_s(long n, const float* a, long lda, int upper, const float* v, double sigma, float* fact)
{
  return upper ? llt_rank_update_run<float, Upper>(n, a, lda, v, sigma, fact)
               : llt_rank_update_run<float, Lower>(n, a, lda, v, sigma, fact);
}

int ref_ldlt_d(long n, const double* a, long lda, int upper, long nrhs, const double* b, long ldb, double* fact,
               int* tr, double* x, double* rcond, int* flags)
{
  return upper ? ldlt_run<double, Upper>(n, a, lda, nrhs, b, ldb, fact, tr, x, rcond, flags)
               : ldlt_run<double, Lower>(n, a, lda, nrhs, b, ldb, fact, tr, x, rcond, flags);
}

int ref_ldlt_s(long n, const float* a, long lda, int upper, long nrhs, const float* b, long ldb, float* fact,
               int* tr, float* x, double* rcond, int* flags)
{
  return upper ? ldlt_run<float, Upper>(n, a, lda, nrhs, b, ldb, fact, tr, x, rcond, flags)
               : ldlt_run<float, Lower>(n, a, lda, nrhs, b, ldb, fact, tr, x, rcond, flags);
}

int ref_llt_d(long n, const double* a, long lda, int upper, long nrhs, const double* b, long ldb, double* fact,
              double* x, double* rcond)
{
  return upper ? llt_run<double, Upper>(n, a, lda, nrhs, b, ldb, fact, x, rcond)
               : llt_run<double, Lower>(n, a, lda, nrhs, b, ldb, fact, x, rcond);
}

int ref_llt_s(long n, const float* a, long lda, int upper, long nrhs, const float* b, long ldb, float* fact,
              float* x, double* rcond)
{
  return upper ? llt_run<float, Upper>(n, a, lda, nrhs, b, ldb, fact, x, rcond)
               : llt_run<float, Lower>(n, a, lda, nrhs, b, ldb, fact, x, rcond);
}

int ref_lu_d(long n, const double* a, long lda, long nrhs, const double* b, long ldb, double* fact, int* perm,
             double* x, double* xt, double* rcond, double* det)
{
  return lu_run<double>(n, a, lda, nrhs, b, ldb, fact, perm, x, xt, rcond, det);
}

int ref_lu_s(long n, const float* a, long lda, long nrhs, const float* b, long ldb, float* fact, int* perm,
             float* x, float* xt, double* rcond, double* det)
{
  return lu_run<float>(n, a, lda, nrhs, b, ldb, fact, perm, x, xt, rcond, det);
}

// The reference's internal blocked kernels, called directly (the functions the
// GPU plug-in replaces): returns the first failing column / zero pivot or -1.
long ref_llt_blocked_d(long n, double* a, long lda)
{
  Map<MatrixXd, 0, OuterStride<> > A(a, n, n, OuterStride<>(lda));
  return internal::llt_inplace<double, Lower>::blocked(A);
}

long ref_lu_blocked_d(long m, long n, double* a, long lda, int* transpositions, int* nb_transpositions)
{
  return internal::partial_lu_impl<double, ColMajor, int>::blocked_lu(m, n, a, lda, transpositions,
                                                                       *nb_transpositions);
}

long ref_lu_blocked_s(long m, long n, float* a, long lda, int* transpositions, int* nb_transpositions)
{
  return internal::partial_lu_impl<float, ColMajor, int>::blocked_lu(m, n, a, lda, transpositions,
                                                                      *nb_transpositions);
}

void ref_set_threads(int t) { Eigen::setNbThreads(t); }
int ref_get_threads(void) { return Eigen::nbThreads(); }

}  // extern "C"
