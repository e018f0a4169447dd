// Test infrastructure, force-included (-include) before the reference's CPU services: the
// CUDA runtime names that src/constants.h and src/services/pst.h mention (an error type, a
// stream handle and the error-string function CUDA_Abort would call). The CPU services
// never call into CUDA; these declarations only let the headers compile without it.
#ifndef ORB_REFSHIM_CUDA_DECLS_H
#define ORB_REFSHIM_CUDA_DECLS_H

#include <cassert>
#include <cstdio>
#include <cstdlib>
#include <cstring>

typedef int cudaError_t;
typedef struct CUstream_st *cudaStream_t;
inline const char *cudaGetErrorString(cudaError_t) { return "CUDA is not used by the CPU services"; }

#endif
