/* See mkl_lapacke.h: the reference build's MKL row is disabled. */
#include "mkl_lapacke.h"
int LAPACKE_sgtsv(int layout, int n, int nrhs, float *dl, float *d, float *du, float *b, int ldb) {
    (void)layout; (void)n; (void)nrhs; (void)dl; (void)d; (void)du; (void)b; (void)ldb;
    return -1;
}
int LAPACKE_dgtsv(int layout, int n, int nrhs, double *dl, double *d, double *du, double *b, int ldb) {
    (void)layout; (void)n; (void)nrhs; (void)dl; (void)d; (void)du; (void)b; (void)ldb;
    return -1;
}
