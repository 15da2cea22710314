// ref_device.cu -- TEST INFRASTRUCTURE: the reference's own device code,
// compiled from its unmodified grid.cu into a device-only fatbin so that the
// reference kernels can run on the GPU machine, where neither its sources nor an
// aarch64 build of its host program exist.
//
// The translation unit includes grid.cu as it lies in the reference tree
// (found through the include path the recipe in oracle/build.py passes) and
// adds extern "C" probe kernels that call the reference's own __device__
// math (signf, minmod, limiter, getVelocity, grid.cu:62-84) on tables of
// inputs.  Those probes pin the limiter semantics on the GPU itself.
//
// Build flags follow the reference CMake: --use_fast_math (CMakeLists.txt:35).

#include "grid.cu"

extern "C" __global__ void ref_probe_signf(const double* a, double* out, int n) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) out[k] = signf(a[k]);
}

extern "C" __global__ void ref_probe_minmod(const double* a, const double* b, const double* c,
                                            double* out, int n) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) out[k] = minmod(a[k], b[k], c[k]);
}

extern "C" __global__ void ref_probe_limiter(const double* u, const double* up1,
                                             const double* um1, double* out, int n) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) out[k] = limiter(u[k], up1[k], um1[k]);
}

extern "C" __global__ void ref_probe_velocity(const double* h, const double* hz, double* out,
                                              int n) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) out[k] = getVelocity(h[k], hz[k]);
}
