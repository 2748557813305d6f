/* Stand-in for Intel MKL's LAPACKE header (MKL is not installed).  Only the
 * two ?gtsv entry points named by Tridiagonal_AVX512/tridiagonal_basic.cpp
 * are declared; lapacke_stub.c makes them fail with -1 so that nothing can
 * mistake the reference build's MKL row for a real LAPACK result. */
#ifndef TRIDIAG_REF_MKL_LAPACKE_H
#define TRIDIAG_REF_MKL_LAPACKE_H
#define LAPACK_COL_MAJOR 102
#ifdef __cplusplus
extern "C" {
#endif
int LAPACKE_sgtsv(int layout, int n, int nrhs, float *dl, float *d, float *du, float *b, int ldb);
int LAPACKE_dgtsv(int layout, int n, int nrhs, double *dl, double *d, double *du, double *b, int ldb);
#ifdef __cplusplus
}
#endif
#endif
