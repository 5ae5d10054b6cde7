/* Thread-control calls that the reference makes only in commented-out code. */
#pragma once
#include "mkl_types.h"
#include "mkl_lapacke.h"
#define MKL_DOMAIN_PARDISO 4
static inline void mkl_set_dynamic(int) {}
static inline void mkl_set_num_threads(int) {}
static inline int mkl_domain_set_num_threads(int, int) { return 0; }
