// Test probe for the integer-pipe conversions of mara2_gb300/csrc/hydro_tile.cuh
// (built by the tests with the fused kernels' flags, not part of the library):
// for each argument, the conversion instruction's result and the integer
// form's, side by side.
#include <cuda_runtime.h>

#include "../mara2_gb300/csrc/hydro_tile.cuh"

__global__ void k_conv(const double* d, const float* f, int n, float* d2f_hw, float* d2f_int, double* f2d_hw,
                       double* f2d_int, double* half_hw, double* half_int)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    d2f_hw[i] = __double2float_rn(d[i]);
    d2f_int[i] = mara::d2f_rn_ftz(d[i]);
    f2d_hw[i] = (double) f[i];
    f2d_int[i] = mara::f2d_exact(f[i]);
    half_hw[i] = __dmul_rn(0.5, d[i]);
    half_int[i] = mara::half_exact(d[i]);
}

// host arrays in, host arrays out; 0 on success
extern "C" int conv_eval(const double* d, const float* f, int n, float* d2f_hw, float* d2f_int, double* f2d_hw,
                         double* f2d_int, double* half_hw, double* half_int)
{
    double *dd = nullptr, *o3 = nullptr, *o4 = nullptr, *o5 = nullptr, *o6 = nullptr;
    float *df = nullptr, *o1 = nullptr, *o2 = nullptr;
    const size_t D = sizeof(double) * (size_t) n, F = sizeof(float) * (size_t) n;
    int rc = 1;
    if (cudaMalloc(&dd, D) == cudaSuccess && cudaMalloc(&df, F) == cudaSuccess && cudaMalloc(&o1, F) == cudaSuccess &&
        cudaMalloc(&o2, F) == cudaSuccess && cudaMalloc(&o3, D) == cudaSuccess && cudaMalloc(&o4, D) == cudaSuccess &&
        cudaMalloc(&o5, D) == cudaSuccess && cudaMalloc(&o6, D) == cudaSuccess) {
        cudaMemcpy(dd, d, D, cudaMemcpyHostToDevice);
        cudaMemcpy(df, f, F, cudaMemcpyHostToDevice);
        k_conv<<<(n + 255) / 256, 256>>>(dd, df, n, o1, o2, o3, o4, o5, o6);
        cudaMemcpy(d2f_hw, o1, F, cudaMemcpyDeviceToHost);
        cudaMemcpy(d2f_int, o2, F, cudaMemcpyDeviceToHost);
        cudaMemcpy(f2d_hw, o3, D, cudaMemcpyDeviceToHost);
        cudaMemcpy(f2d_int, o4, D, cudaMemcpyDeviceToHost);
        cudaMemcpy(half_hw, o5, D, cudaMemcpyDeviceToHost);
        cudaMemcpy(half_int, o6, D, cudaMemcpyDeviceToHost);
        rc = cudaDeviceSynchronize() == cudaSuccess ? 0 : 1;
    }
    cudaFree(dd); cudaFree(df); cudaFree(o1); cudaFree(o2); cudaFree(o3); cudaFree(o4); cudaFree(o5); cudaFree(o6);
    return rc;
}
