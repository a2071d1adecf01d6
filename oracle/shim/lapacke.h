/* Test infrastructure (oracle): LAPACKE subset referenced by the reference's
 * linalg.hpp.  getrf/getrs/zgetrs are implemented by the project's partial-
 * pivoting LU (shim_impl.cpp), which follows LAPACK's unblocked dgetf2 order:
 * pivot = first entry of maximal magnitude in the column, row swap, scale,
 * rank-1 update.  The Cholesky routines are declared only (never called). */
#pragma once
#include <complex>
typedef int lapack_int;
typedef std::complex<double> lapack_complex_double;
#define LAPACK_COL_MAJOR 102
#define LAPACK_ROW_MAJOR 101
lapack_int LAPACKE_dgetrf(int layout, lapack_int m, lapack_int n, double *a, lapack_int lda, lapack_int *ipiv);
lapack_int LAPACKE_dgetrs(int layout, char trans, lapack_int n, lapack_int nrhs, const double *a, lapack_int lda,
                          const lapack_int *ipiv, double *b, lapack_int ldb);
lapack_int LAPACKE_zgetrs(int layout, char trans, lapack_int n, lapack_int nrhs, const lapack_complex_double *a,
                          lapack_int lda, const lapack_int *ipiv, lapack_complex_double *b, lapack_int ldb);
lapack_int LAPACKE_dpotrf(int layout, char uplo, lapack_int n, double *a, lapack_int lda);
lapack_int LAPACKE_dpotrs(int layout, char uplo, lapack_int n, lapack_int nrhs, const double *a, lapack_int lda,
                          double *b, lapack_int ldb);
lapack_int LAPACKE_zpotrs(int layout, char uplo, lapack_int n, lapack_int nrhs, const lapack_complex_double *a,
                          lapack_int lda, lapack_complex_double *b, lapack_int ldb);
