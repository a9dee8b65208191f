// diagnostics.cuh -- device diagnostics of a resident state, shared by the
// plain (diagnostics.cu) and mixed (mixed.cu) paths.
//
// volume diagnostics: FieldOperator::volumeIntegratedDiagnostics
// (FieldOperator.cpp:171-205): per interior zone, ConservationLaw::
// makeDiagnostics of fromPrimitive(P) with the default request (area element
// x-hat, ConservationLaws.cpp:146-157), times the cell volume, summed.  Each
// block sums its zones in a fixed order and writes one partial per
// diagnostic; one more block adds the partials in block order, so the result
// is the same on every run.  The sum order differs from the reference's
// sequential loop, so totals agree to rounding, not bit for bit.
//
// field diagnostics: CellCenteredFieldCT::monopole and ::current with
// MeshLocation::cell (CellCenteredFieldCT.cpp:159-257) at every cell of the
// array with guards, as the reference's checkpoint task stores them in
// MeshData's diagnostic fields (src/Problems/MagneticBraiding.cpp:176-189).
#pragma once

#include "physics_fp64.cuh"

namespace mara {

constexpr int DIAG_MAX = 18;
constexpr int DIAG_BLOCKS = 1024;  // partial sums per reduction

template <int LAW> struct DiagInfo {
    static constexpr int ND = LAW == LAW_HYDRO ? 5 : LAW == LAW_MHD_COOL ? 18 : 17;
};

// ConservationLaw::makeDiagnostics: NewtonianHydro ConservationLaws.cpp:
// 321-330, NewtonianMHD :536-574 (with the cooling auxiliary field), RelativisticMHD
// :874-922
template <int LAW>
__device__ __forceinline__ int make_diagnostics(const PhysParams& pp, const double* P, double* D)
{
    constexpr int NQ = LawInfo<LAW>::NQ;
    double U[NQ];
    const int e = law_p2u<LAW>(pp, P, U);
    if (e != ST_OK) return e;
    if constexpr (LAW == LAW_HYDRO) {
#pragma unroll
        for (int q = 0; q < 5; ++q) D[q] = U[q];
    } else {
        const double gm = pp.gamma;
        const double vv = P[1] * P[1] + P[2] * P[2] + P[3] * P[3];
        const double BB = P[5] * P[5] + P[6] * P[6] + P[7] * P[7];
        const double Bv = P[5] * P[1] + P[6] * P[2] + P[7] * P[3];
        const double cs = sqrt(gm * P[4] / P[0]);
        const double ca = sqrt(BB / P[0]);
        const double s0 = P[4] / pow(P[0], gm);
        const double Ms = sqrt(vv) / cs;
        const double Ma = sqrt(vv) / ca;
#pragma unroll
        for (int q = 0; q < 8; ++q) D[q] = U[q];
        if constexpr (LAW == LAW_MHD || LAW == LAW_MHD_COOL) {
            D[8] = 0.5 * vv * P[0];
            D[9] = P[4] / (gm - 1.0);
            D[10] = 0.5 * BB;
        } else {
            const double E1 = -(P[2] * P[7] - P[3] * P[6]);
            const double E2 = -(P[3] * P[5] - P[1] * P[7]);
            const double E3 = -(P[1] * P[6] - P[2] * P[5]);
            const double EE = (E1 * E1 + E2 * E2 + E3 * E3);
            const double g0 = 1.0 / sqrt(1 - vv);
            const double d0 = P[0];
            const double p0 = P[4];
            const double e0 = p0 / d0 / (gm - 1);
            const double h0 = 1.0 + e0 + p0 / d0;
            D[8] = g0 * (g0 - 1) * d0 * h0;
            D[9] = p0 * (g0 - 1) + d0 * e0 * g0;
            D[10] = 0.5 * (BB + EE);
        }
        D[11] = cs;
        D[12] = ca;
        D[13] = Ms;
        D[14] = Ma;
        D[15] = s0;
        D[16] = Bv;
        if constexpr (LAW == LAW_MHD_COOL) D[17] = U[8];  // the auxiliary field
    }
    return ST_OK;
}

// Src::load(i, j, k, P) fills the primitive state of interior zone (i, j, k)
// and returns a status.
template <int LAW, class Src>
__global__ void __launch_bounds__(256) k_volume_diag(Src src, PhysParams pp, int n0, int n1, long long zones,
                                                     double dV, double* __restrict__ partial, int* __restrict__ err)
{
    constexpr int ND = DiagInfo<LAW>::ND;
    constexpr int NQ = LawInfo<LAW>::NQ;
    double acc[ND];
#pragma unroll
    for (int n = 0; n < ND; ++n) acc[n] = 0.0;
    for (long long z = blockIdx.x * (long long) blockDim.x + threadIdx.x; z < zones;
         z += (long long) gridDim.x * blockDim.x) {
        const int i = (int) (z % n0);
        const int j = (int) ((z / n0) % n1);
        const int k = (int) (z / ((long long) n0 * n1));
        double P[NQ], D[ND];
        int e = src.load(i, j, k, P);
        if (e == ST_OK) e = make_diagnostics<LAW>(pp, P, D);
        if (e != ST_OK) {
            atomicCAS(err, 0, e);
            continue;
        }
#pragma unroll
        for (int n = 0; n < ND; ++n) acc[n] += D[n] * dV;
    }
    __shared__ double red[ND][8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int n = 0; n < ND; ++n) {
        double v = acc[n];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
        if (lane == 0) red[n][warp] = v;
    }
    __syncthreads();
    if (threadIdx.x < ND) {
        double v = 0.0;
        for (int w = 0; w < (int) (blockDim.x >> 5); ++w) v += red[threadIdx.x][w];
        partial[blockIdx.x * ND + threadIdx.x] = v;
    }
}

static __global__ void k_diag_final(const double* __restrict__ partial, int nblocks, int nd, double* __restrict__ out)
{
    const int n = threadIdx.x;
    if (n >= nd) return;
    double v = 0.0;
    for (int b = 0; b < nblocks; ++b) v += partial[b * nd + n];
    out[n] = v;
}

// cell field B of cell (i, j, k) of the array with guards (N0, N1, N2), SoA
// with the field components at 5, 6, 7 as the primitive arrays hold them
template <typename T>
struct CellB {
    const T* P;
    long long sP;
    int N0, N1, N2;
    __device__ __forceinline__ double operator()(int i, int j, int k, int c) const
    {
        return (double) P[(5 + c) * sP + ((long long) k * N1 + j) * N0 + i];
    }
};

// vertex monopole M(a, b, c) of CellCenteredFieldCT::monopole: the reference
// fills M(i+1, j+1, k+1) for i < N0 - r (and so on) and leaves the rest 0
template <typename T>
__device__ __forceinline__ double vertex_monopole_at(const CellB<T>& B, int a, int b, int c, double h)
{
    const int r = B.N0 > 1, s = B.N1 > 1, t = B.N2 > 1;
    const int i = a - 1, j = b - 1, k = c - 1;
    if (i < 0 || j < 0 || k < 0 || i >= B.N0 - r || j >= B.N1 - s || k >= B.N2 - t) return 0.0;
    const double Bx0 = B(i, j, k, 0) + B(i, j, k + t, 0) + B(i, j + s, k, 0) + B(i, j + s, k + t, 0);
    const double Bx1 = B(i + r, j, k, 0) + B(i + r, j, k + t, 0) + B(i + r, j + s, k, 0) + B(i + r, j + s, k + t, 0);
    const double By0 = B(i, j, k, 1) + B(i + r, j, k, 1) + B(i, j, k + t, 1) + B(i + r, j, k + t, 1);
    const double By1 = B(i, j + s, k, 1) + B(i + r, j + s, k, 1) + B(i, j + s, k + t, 1) + B(i + r, j + s, k + t, 1);
    const double Bz0 = B(i, j, k, 2) + B(i, j + s, k, 2) + B(i + r, j, k, 2) + B(i + r, j + s, k, 2);
    const double Bz1 = B(i, j, k + t, 2) + B(i, j + s, k + t, 2) + B(i + r, j, k + t, 2) + B(i + r, j + s, k + t, 2);
    return 0.25 * ((Bx1 - Bx0) + (By1 - By0) + (Bz1 - Bz0)) / h;
}

// out (N0, N1, N2, 4) AoS, C order: [monopole, current1, current2, current3]
template <typename T>
__global__ void __launch_bounds__(256) k_field_diag(CellB<T> B, double h, double* __restrict__ out)
{
    const long long total = (long long) B.N0 * B.N1 * B.N2;
    const long long c = blockIdx.x * (long long) blockDim.x + threadIdx.x;
    if (c >= total) return;
    // AoS cell index, k fastest
    const int k = (int) (c % B.N2);
    const int j = (int) ((c / B.N2) % B.N1);
    const int i = (int) (c / ((long long) B.N2 * B.N1));
    const double M000 = vertex_monopole_at(B, i, j, k, h);
    const double Mi = M000 + vertex_monopole_at(B, i + 1, j, k, h);
    const double Mj = M000 + vertex_monopole_at(B, i, j + 1, k, h);
    const double Mk = M000 + vertex_monopole_at(B, i, j, k + 1, h);
    double J[3] = {0.0, 0.0, 0.0};
    const int r = B.N0 > 1, s = B.N1 > 1, t = B.N2 > 1;
    const int a = i - r, b = j - s, e = k - t;  // the reference's loop index
    if (a >= 0 && b >= 0 && e >= 0 && a < B.N0 - 2 * r && b < B.N1 - 2 * s && e < B.N2 - 2 * t) {
        const double d0B1 = B(a + 2 * r, b, e, 1) - B(a, b, e, 1);
        const double d0B2 = B(a + 2 * r, b, e, 2) - B(a, b, e, 2);
        const double d1B2 = B(a, b + 2 * s, e, 2) - B(a, b, e, 2);
        const double d1B0 = B(a, b + 2 * s, e, 0) - B(a, b, e, 0);
        const double d2B0 = B(a, b, e + 2 * t, 0) - B(a, b, e, 0);
        const double d2B1 = B(a, b, e + 2 * t, 1) - B(a, b, e, 1);
        J[0] = (d1B2 - d2B1) / h / 2;
        J[1] = (d2B0 - d0B2) / h / 2;
        J[2] = (d0B1 - d1B0) / h / 2;
    }
    out[c * 4 + 0] = 1. / 6 * (Mi + Mj + Mk);
    out[c * 4 + 1] = J[0];
    out[c * 4 + 2] = J[1];
    out[c * 4 + 3] = J[2];
}

} // namespace mara
