// Minimal stand-in for the CUDA samples' helper_cuda.h, which the reference
// includes (grid.cu:6) but does not ship.  Only what grid.cu needs to compile
// its device code: checkCudaErrors and the std headers it relies on.
#pragma once
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>
#include <cuda_runtime.h>
#define checkCudaErrors(call)                                                      \
    do {                                                                           \
        cudaError_t e_ = (call);                                                   \
        if (e_ != cudaSuccess) {                                                   \
            std::fprintf(stderr, "CUDA error %s at %s:%d\n", cudaGetErrorString(e_), \
                         __FILE__, __LINE__);                                      \
            std::exit(1);                                                          \
        }                                                                          \
    } while (0)
