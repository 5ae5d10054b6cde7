/* PARDISO entry points used by the reference (calMatrixOperations.cpp:255-376). */
#pragma once
#include "mkl_types.h"
void PARDISO_64(void* pt, const long long* maxfct, const long long* mnum, const long long* mtype,
                const long long* phase, const long long* n, const double* a, const long long* ia,
                const long long* ja, long long* perm, const long long* nrhs, long long* iparm,
                const long long* msglvl, double* b, double* x, long long* error);
