/* MKL type names used by the reference, built with -DMKL_ILP64 (64-bit ints). */
#pragma once
typedef long long MKL_INT;
