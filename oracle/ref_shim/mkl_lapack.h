/* Empty stand-in for Intel MKL's mkl_lapack.h (see mkl_lapacke.h). */
