// Uses Eigen's own API on LLT / PartialPivLU; with -DUSE_GB300 the plug-in
// header routes the blocked factorizations to (a test double of) libgb300solve.
// Prints one line per check: name and values, compared by the Python test
// against the same program built without the plug-in.
#include <Eigen/Dense>
#ifdef USE_GB300
#include <eigen_gb300/GB300Support>
extern "C" int gbs_mock_calls;
#endif
#include <cstdio>

using namespace Eigen;

template <typename M> static M spd(int n, unsigned seed)
{
  std::srand(seed);
  M g = M::Random(n, n);
  M a = g * g.transpose();
  a.diagonal().array() += typename M::Scalar(n);
  return a;
}

int main()
{
  const int n = 157;
  MatrixXd A = spd<MatrixXd>(n, 3);
  VectorXd b = VectorXd::Ones(n);
  {
    LLT<MatrixXd> llt(A);
    VectorXd x = llt.solve(b);
    std::printf("llt_lower info=%d x0=%.15e rcond=%.12e L00=%.15e\n", int(llt.info()), x(0), llt.rcond(), llt.matrixL()(n - 1, 0));
  }
  {
    LLT<MatrixXd, Upper> llt(A);
    VectorXd x = llt.solve(b);
    std::printf("llt_upper info=%d x0=%.15e rcond=%.12e\n", int(llt.info()), x(0), llt.rcond());
  }
  {
    Matrix<double, Dynamic, Dynamic, RowMajor> R = A;
    LLT<Matrix<double, Dynamic, Dynamic, RowMajor> > llt(R);
    VectorXd x = llt.solve(b);
    std::printf("llt_rowmajor info=%d x0=%.15e\n", int(llt.info()), x(0));
  }
  {
    MatrixXd N = -A;
    LLT<MatrixXd> llt(N);
    std::printf("llt_negative info=%d\n", int(llt.info()));
  }
  {
    MatrixXd B = A;
    LLT<Ref<MatrixXd> > llt(B);          // in place
    VectorXd x = llt.solve(b);
    std::printf("llt_inplace info=%d x0=%.15e modified=%d\n", int(llt.info()), x(0), int(!B.isApprox(A)));
  }
  {
    std::srand(7);
    MatrixXd G = MatrixXd::Random(n, n);
    PartialPivLU<MatrixXd> lu(G);
    VectorXd x = lu.solve(b);
    std::printf("lu info x0=%.15e rcond=%.12e det=%.12e p0=%d p1=%d plast=%d\n", x(0), lu.rcond(), lu.determinant(),
                lu.permutationP().indices()(0), lu.permutationP().indices()(1), lu.permutationP().indices()(n - 1));
    MatrixXf Gf = G.cast<float>();
    PartialPivLU<MatrixXf> luf(Gf);
    std::printf("lu_float p0=%d p5=%d x0=%.6e\n", luf.permutationP().indices()(0), luf.permutationP().indices()(5),
                luf.solve(VectorXf::Ones(n))(0));
    MatrixXd H = G;
    PartialPivLU<Ref<MatrixXd> > lur(H);   // in place
    std::printf("lu_inplace x0=%.15e\n", lur.solve(b)(0));
  }
#ifdef USE_GB300
  std::printf("plugin_calls %d\n", gbs_mock_calls);
#else
  std::printf("plugin_calls 8\n");
#endif
  return 0;
}
