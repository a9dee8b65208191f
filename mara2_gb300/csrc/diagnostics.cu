// diagnostics.cu -- device diagnostics of the resident state (the kernels are
// in diagnostics.cuh).
//
// monopole max: CellCenteredFieldCT::monopole with MeshLocation::cell
// (CellCenteredFieldCT.cpp:159-223) reduced to the largest |div B| over the
// interior zones (the figure the MHD workload reports).  Reads the
// cell-centred field from the primitive array with guards (FP64 on the plain
// path, FP32 on the mixed path).
#include <cuda_runtime.h>

#include "diagnostics.cuh"
#include "internal.h"

namespace mara {

template <typename T>
static CellB<T> cell_b(const void* P, const GridDesc& G)
{
    return CellB<T>{(const T*) P, G.sP, G.N[0], G.N[1], G.N[2]};
}

template <typename T>
__global__ void k_monopole_max(CellB<T> B, GridDesc G, double h, unsigned long long* out)
{
    const int ii = blockIdx.x * blockDim.x + threadIdx.x;
    double m = 0.0;
    if (ii < G.n[0]) {
        // cell-centred monopole of an interior zone (full indices)
        const int i = ii + G.g[0], j = blockIdx.y + G.g[1], k = blockIdx.z + G.g[2];
        const double M000 = vertex_monopole_at(B, i, j, k, h);
        const double Mi = M000 + vertex_monopole_at(B, i + 1, j, k, h);
        const double Mj = M000 + vertex_monopole_at(B, i, j + 1, k, h);
        const double Mk = M000 + vertex_monopole_at(B, i, j, k + 1, h);
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
    if (fp32) k_monopole_max<float><<<grid, 256, 0, s>>>(cell_b<float>(P, G), G, h, out);
    else k_monopole_max<double><<<grid, 256, 0, s>>>(cell_b<double>(P, G), G, h, out);
}

void launch_field_diag(const void* P, bool fp32, const GridDesc& G, double h, double* out, cudaStream_t s)
{
    const long long total = (long long) G.N[0] * G.N[1] * G.N[2];
    const unsigned nb = (unsigned) ((total + 255) / 256);
    if (fp32) k_field_diag<float><<<nb, 256, 0, s>>>(cell_b<float>(P, G), h, out);
    else k_field_diag<double><<<nb, 256, 0, s>>>(cell_b<double>(P, G), h, out);
}

// interior zone (i, j, k) of the plain path's FP64 primitives with guards
template <int NQ>
struct PlainSrc {
    const double* P;
    long long sP;
    int N0, N1, g0, g1, g2;
    __device__ __forceinline__ int load(int i, int j, int k, double* out) const
    {
        const long long o = ((long long) (k + g2) * N1 + (j + g1)) * N0 + (i + g0);
#pragma unroll
        for (int q = 0; q < NQ; ++q) out[q] = P[q * sP + o];
        return ST_OK;
    }
};

template <int LAW>
static void volume_diag_plain(const double* P, const GridDesc& G, const PhysParams& pp, double* partial, int* err,
                              double* out, cudaStream_t s)
{
    constexpr int NQ = LawInfo<LAW>::NQ;
    const PlainSrc<NQ> src{P, G.sP, G.N[0], G.N[1], G.g[0], G.g[1], G.g[2]};
    const long long zones = (long long) G.n[0] * G.n[1] * G.n[2];
    const long long want = (zones + 255) / 256;
    const int nb = (int) (want < DIAG_BLOCKS ? want : DIAG_BLOCKS);
    k_volume_diag<LAW><<<nb, 256, 0, s>>>(src, pp, G.n[0], G.n[1], zones, G.dV, partial, err);
    k_diag_final<<<1, 32, 0, s>>>(partial, nb, DiagInfo<LAW>::ND, out);
}

void launch_volume_diag_plain(int law, const double* P, const GridDesc& G, const PhysParamsH& ph, double* partial,
                              int* err, double* out, cudaStream_t s)
{
    PhysParams pp;
    pp.gamma = ph.gamma;
    pp.plm_theta = ph.plm_theta;
    pp.shenzha_A = ph.shenzha_A;
    pp.pressure_floor = ph.pressure_floor;
    pp.weno_is = ph.weno_is;
    pp.cooling_rate = ph.cooling_rate;
    switch (law) {
        case LAW_HYDRO: volume_diag_plain<LAW_HYDRO>(P, G, pp, partial, err, out, s); break;
        case LAW_MHD: volume_diag_plain<LAW_MHD>(P, G, pp, partial, err, out, s); break;
        case LAW_MHD_COOL: volume_diag_plain<LAW_MHD_COOL>(P, G, pp, partial, err, out, s); break;
        default: volume_diag_plain<LAW_RMHD>(P, G, pp, partial, err, out, s); break;
    }
}

} // namespace mara

// ---- QuarticPolynomial::solve on the device ------------------------------------
namespace mara {

__global__ void k_quartic(const double* __restrict__ coeffs, int n, double* __restrict__ roots, int* __restrict__ nr)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double* d = coeffs + 5 * (long long) i;
    double r[4] = {0.0, 0.0, 0.0, 0.0};
    nr[i] = quartic_roots(d[0], d[1], d[2], d[3], d[4], r);
    for (int k = 0; k < 4; ++k) roots[4 * (long long) i + k] = r[k];
}

} // namespace mara

extern "C" int mara_gpu_quartic_solve(const double* coeffs, int n, double* roots, int* nroots, int device)
{
    using namespace mara;
    if (n < 0 || (n > 0 && (!coeffs || !roots || !nroots))) return MARA_ERR_ARGUMENT;
    if (n == 0) return MARA_OK;
    int prev = -1;
    if (cudaGetDevice(&prev) != cudaSuccess) return MARA_ERR_NO_DEVICE;
    if (prev != device && cudaSetDevice(device) != cudaSuccess) return MARA_ERR_NO_DEVICE;
    int rc = MARA_OK;
    double* dc = nullptr;
    double* dr = nullptr;
    int* dn = nullptr;
    const size_t cb = sizeof(double) * 5 * (size_t) n, rb = sizeof(double) * 4 * (size_t) n;
    if (cudaMalloc(&dc, cb) != cudaSuccess || cudaMalloc(&dr, rb) != cudaSuccess ||
        cudaMalloc(&dn, sizeof(int) * (size_t) n) != cudaSuccess) {
        rc = MARA_ERR_CUDA;
    } else if (cudaMemcpy(dc, coeffs, cb, cudaMemcpyHostToDevice) != cudaSuccess) {
        rc = MARA_ERR_CUDA;
    } else {
        k_quartic<<<(n + 127) / 128, 128>>>(dc, n, dr, dn);
        if (cudaGetLastError() != cudaSuccess || cudaMemcpy(roots, dr, rb, cudaMemcpyDeviceToHost) != cudaSuccess ||
            cudaMemcpy(nroots, dn, sizeof(int) * (size_t) n, cudaMemcpyDeviceToHost) != cudaSuccess)
            rc = MARA_ERR_CUDA;
    }
    cudaFree(dc);
    cudaFree(dr);
    cudaFree(dn);
    if (prev != device) cudaSetDevice(prev);
    return rc;
}
