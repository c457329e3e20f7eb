// ORACLE / TEST INFRASTRUCTURE — header shim that lets the unmodified Veritas sources
// build in their default configuration (CMakeLists.txt:9 `USE_MKL ON`, which defines
// USINGMKL and MKL_ILP64) without Intel MKL.  Only the four MKL routines the sources
// call are declared:
//   LAPACKE_dgetrf / LAPACKE_dgetrs  (EMSolver.cpp:75, EMSolver.cpp:177)
//   vdLn                             (Rectangle.cpp:227-229, moments)
//   vdExp                            (only referenced under MKLINIT==1, which is 0)
// They are implemented in mkl_shim.cpp: the LU is the fill-aware exact restatement in
// oracle/lu_exact.hpp; vdLn/vdExp apply std::log / std::exp element by element.
#pragma once
#include <cstdint>
typedef long long lapack_int;
#define LAPACK_ROW_MAJOR 101
#define LAPACK_COL_MAJOR 102
lapack_int LAPACKE_dgetrf(int matrix_layout, lapack_int m, lapack_int n, double *a, lapack_int lda, lapack_int *ipiv);
lapack_int LAPACKE_dgetrs(int matrix_layout, char trans, lapack_int n, lapack_int nrhs, const double *a, lapack_int lda,
                          const lapack_int *ipiv, double *b, lapack_int ldb);
void vdLn(lapack_int n, const double *a, double *r);
void vdExp(lapack_int n, const double *a, double *r);
