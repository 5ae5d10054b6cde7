/* LAPACKE entry points used by the reference (calMatrixOperations.cpp:616,660).
 * Implemented in shim_impl.cpp on top of a LAPACK found at build time. */
#pragma once
#include "mkl_types.h"
#define LAPACK_ROW_MAJOR 101
#define LAPACK_COL_MAJOR 102
MKL_INT LAPACKE_dgesv(int layout, MKL_INT n, MKL_INT nrhs, double* a, MKL_INT lda,
                      MKL_INT* ipiv, double* b, MKL_INT ldb);
MKL_INT LAPACKE_dsyev(int layout, char jobz, char uplo, MKL_INT n, double* a,
                      MKL_INT lda, double* w);
