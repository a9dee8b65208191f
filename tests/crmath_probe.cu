// Test probe for mara2_gb300/csrc/crmath.cuh (built by the tests, not part
// of the library).  fn: 0 pow(x, 1/3), 1 acos, 2 cos, 3 sin.
//
// host_eval: the host's libm and crmath's evaluation compiled for the host.
// dev_eval (nvcc builds only): CUDA's own function and crmath's evaluation
// on the device, for the same arguments.
#include <math.h>
#include <stdlib.h>

#include "../mara2_gb300/csrc/crmath.cuh"

extern "C" void host_eval(int fn, const double* x, int n, double* libm, double* cr)
{
    for (int i = 0; i < n; ++i) {
        const double v = x[i];
        switch (fn) {
            case 0: libm[i] = pow(v, 1. / 3); cr[i] = crm::pow_third(v); break;
            case 1: libm[i] = acos(v); cr[i] = crm::acos_cr(v); break;
            case 2: libm[i] = cos(v); cr[i] = crm::cos_cr(v); break;
            default: libm[i] = sin(v); cr[i] = crm::sin_cr(v); break;
        }
    }
}

#if defined(__CUDACC__)
#include <cuda_runtime.h>

__global__ void k_eval(int fn, const double* x, int n, double* lib, double* cr)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double v = x[i];
    switch (fn) {
        case 0: lib[i] = pow(v, 1. / 3); cr[i] = crm::pow_third(v); break;
        case 1: lib[i] = acos(v); cr[i] = crm::acos_cr(v); break;
        case 2: lib[i] = cos(v); cr[i] = crm::cos_cr(v); break;
        default: lib[i] = sin(v); cr[i] = crm::sin_cr(v); break;
    }
}

extern "C" int dev_eval(int fn, const double* x, int n, double* lib, double* cr)
{
    double *dx = nullptr, *dl = nullptr, *dc = nullptr;
    const size_t b = sizeof(double) * (size_t) n;
    int rc = 0;
    if (cudaMalloc(&dx, b) || cudaMalloc(&dl, b) || cudaMalloc(&dc, b)) rc = 1;
    else if (cudaMemcpy(dx, x, b, cudaMemcpyHostToDevice)) rc = 2;
    else {
        k_eval<<<(n + 255) / 256, 256>>>(fn, dx, n, dl, dc);
        if (cudaGetLastError() || cudaMemcpy(lib, dl, b, cudaMemcpyDeviceToHost) ||
            cudaMemcpy(cr, dc, b, cudaMemcpyDeviceToHost))
            rc = 3;
    }
    cudaFree(dx);
    cudaFree(dl);
    cudaFree(dc);
    return rc;
}
#endif
