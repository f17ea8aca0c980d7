// Test infrastructure: compiles the reference's own BLAS level-3 shim
// (blas/level3_impl.h: ?gemm_, ?trsm_, ?syrk_ and the rest of level 3) from the
// read-only reference tree, once per scalar type, into oracle/_ref/.  The tests
// use it as the oracle of the library's gbs_?gemm / gbs_?trsm / gbs_?syrk.
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

#include "level3_impl.h"
