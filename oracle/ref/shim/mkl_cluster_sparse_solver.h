/* cluster_sparse_solver_64 as called by calMatrixOperations.cpp:443-497. */
#pragma once
#include "mkl_types.h"
void cluster_sparse_solver_64(void* pt, const long long* maxfct, const long long* mnum,
                              const long long* mtype, const long long* phase, const long long* n,
                              const double* a, const long long* ia, const long long* ja,
                              long long* perm, const long long* nrhs, long long* iparm,
                              const long long* msglvl, double* b, double* x, const int* comm,
                              long long* error);
