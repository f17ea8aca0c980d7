// Test infrastructure: compiles the reference's own LAPACK C-ABI shim
// (lapack/cholesky.cpp, lapack/lu.cpp: ?potrf_, ?potrs_, ?getrf_, ?getrs_) from
// the read-only reference tree, once per scalar type, into oracle/_ref/.  The
// tests use it to pin the semantics (1-based ipiv, info codes) of the
// library's gbs_?getrf / gbs_?potrf entry points.
#if defined(GB_REF_DOUBLE)
#define SCALAR double
#define SCALAR_SUFFIX d
#define SCALAR_SUFFIX_UP "D"
#elif defined(GB_REF_SINGLE)
#define SCALAR float
#define SCALAR_SUFFIX s
#define SCALAR_SUFFIX_UP "S"
#endif
#define ISCOMPLEX 0

#include "cholesky.cpp"
#include "lu.cpp"
