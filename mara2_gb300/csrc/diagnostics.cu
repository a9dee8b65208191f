// diagnostics.cu -- device diagnostics of the resident state.
//
// monopole: CellCenteredFieldCT::monopole with MeshLocation::cell
// (CellCenteredFieldCT.cpp:159-223): div B at the mesh vertices from the 8
// cells around each vertex, then averaged onto cells; reduced here to the
// largest |div B| over the interior zones (the figure the MHD workload
// reports).  Reads the cell-centred field from the primitive array with
// guards (FP64 on the plain path, FP32 on the mixed path).
#include <cuda_runtime.h>

#include "internal.h"

namespace mara {

template <typename T>
__device__ __forceinline__ double vertex_monopole(const T* __restrict__ P, const GridDesc& G, int a, int b, int c,
                                                  double h)
{
    // vertex (a, b, c) sits at the low corner of cell (a, b, c); the
    // reference writes M(i+1, j+1, k+1) from cells (i..i+r, j..j+s, k..k+t)
    const int r = G.N[0] > 1, s = G.N[1] > 1, t = G.N[2] > 1;
    const int i = a - 1, j = b - 1, k = c - 1;
    if (i < 0 || j < 0 || k < 0 || i >= G.N[0] - r || j >= G.N[1] - s || k >= G.N[2] - t) return 0.0;
    auto B = [&](int ii, int jj, int kk, int comp) -> double {
        return (double) P[(5 + comp) * G.sP + ((long long) kk * G.N[1] + jj) * G.N[0] + ii];
    };
    const double Bx0 = B(i, j, k, 0) + B(i, j, k + t, 0) + B(i, j + s, k, 0) + B(i, j + s, k + t, 0);
    const double Bx1 = B(i + r, j, k, 0) + B(i + r, j, k + t, 0) + B(i + r, j + s, k, 0) + B(i + r, j + s, k + t, 0);
    const double By0 = B(i, j, k, 1) + B(i + r, j, k, 1) + B(i, j, k + t, 1) + B(i + r, j, k + t, 1);
    const double By1 = B(i, j + s, k, 1) + B(i + r, j + s, k, 1) + B(i, j + s, k + t, 1) + B(i + r, j + s, k + t, 1);
    const double Bz0 = B(i, j, k, 2) + B(i, j + s, k, 2) + B(i + r, j, k, 2) + B(i + r, j + s, k, 2);
    const double Bz1 = B(i, j, k + t, 2) + B(i, j + s, k + t, 2) + B(i + r, j, k + t, 2) + B(i + r, j + s, k + t, 2);
    return 0.25 * ((Bx1 - Bx0) + (By1 - By0) + (Bz1 - Bz0)) / h;
}

template <typename T>
__global__ void k_monopole_max(const T* __restrict__ P, GridDesc G, double h, unsigned long long* out)
{
    const int ii = blockIdx.x * blockDim.x + threadIdx.x;
    double m = 0.0;
    if (ii < G.n[0]) {
        // cell-centred monopole of an interior zone (full indices)
        const int i = ii + G.g[0], j = blockIdx.y + G.g[1], k = blockIdx.z + G.g[2];
        const double M000 = vertex_monopole(P, G, i, j, k, h);
        const double Mi = M000 + vertex_monopole(P, G, i + 1, j, k, h);
        const double Mj = M000 + vertex_monopole(P, G, i, j + 1, k, h);
        const double Mk = M000 + vertex_monopole(P, G, i, j, k + 1, h);
        m = fabs(1. / 6 * (Mi + Mj + Mk));
    }
    unsigned long long b = (unsigned long long) __double_as_longlong(m);
    if (!(m >= 0.0)) b = 0x7ff0000000000000ull;  // NaN reports as +inf
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const unsigned long long o = __shfl_down_sync(0xffffffffu, b, off);
        b = o > b ? o : b;
    }
    if ((threadIdx.x & 31) == 0) atomicMax(out, b);
}

void launch_monopole_max(const void* P, bool fp32, const GridDesc& G, double h, unsigned long long* out,
                         cudaStream_t s)
{
    dim3 grid((G.n[0] + 255) / 256, G.n[1], G.n[2]);
    if (fp32) k_monopole_max<float><<<grid, 256, 0, s>>>((const float*) P, G, h, out);
    else k_monopole_max<double><<<grid, 256, 0, s>>>((const double*) P, G, h, out);
}

} // namespace mara
