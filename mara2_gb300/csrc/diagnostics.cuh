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

// Cell monopoles of a tile of cells from its vertex monopoles formed once:
// a cell's value is 1/6 (3 M000 + M(i+1) + M(j+1) + M(k+1)) of four vertex
// monopoles (CellCenteredFieldCT.cpp:200-219), and a vertex is shared by the
// cells around it, so a block first fills the (TX+1) x (TY+1) x (TZ+1) vertex
// monopoles of its TX x TY x TZ cells into shared memory (the same
// vertex_monopole_at values, so the same bits as forming them per cell).
// Tiles: 32 x 8 x 4 cells in 3-D, 32 x 32 x 1 in 2-D; 256 threads.
template <int TZ> struct MonoTile {
    static constexpr int TX = 32, TY = TZ > 1 ? 8 : 32;
    static constexpr int NV = (TX + 1) * (TY + 1) * (TZ + 1);
};

template <typename T, int TZ>
__device__ __forceinline__ void fill_vertex_monopoles(const CellB<T>& B, int a0, int b0, int c0, double h,
                                                      double (*Mv)[MonoTile<TZ>::TY + 1][MonoTile<TZ>::TX + 1])
{
    constexpr int TX = MonoTile<TZ>::TX, TY = MonoTile<TZ>::TY;
    for (int v = threadIdx.x; v < MonoTile<TZ>::NV; v += blockDim.x) {
        const int x = v % (TX + 1), y = (v / (TX + 1)) % (TY + 1), z = v / ((TX + 1) * (TY + 1));
        Mv[z][y][x] = vertex_monopole_at(B, a0 + x, b0 + y, c0 + z, h);
    }
}

// out (N0, N1, N2, 4) AoS, C order: [monopole, current1, current2, current3]
template <typename T, int TZ>
__global__ void __launch_bounds__(256) k_field_diag_tiled(CellB<T> B, double h, double* __restrict__ out)
{
    constexpr int TX = MonoTile<TZ>::TX, TY = MonoTile<TZ>::TY;
    __shared__ double Mv[TZ + 1][TY + 1][TX + 1];
    const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY, k0 = blockIdx.z * TZ;
    fill_vertex_monopoles<T, TZ>(B, i0, j0, k0, h, Mv);
    __syncthreads();
    const int r = B.N0 > 1, s = B.N1 > 1, t = B.N2 > 1;
    // cells of the tile with k fastest, as the AoS output runs
    for (int c = threadIdx.x; c < TX * TY * TZ; c += blockDim.x) {
        const int z = c % TZ, x = (c / TZ) % TX, y = c / (TZ * TX);
        const int i = i0 + x, j = j0 + y, k = k0 + z;
        if (i >= B.N0 || j >= B.N1 || k >= B.N2) continue;
        const double M000 = Mv[z][y][x];
        const double Mi = M000 + Mv[z][y][x + 1];
        const double Mj = M000 + Mv[z][y + 1][x];
        const double Mk = M000 + Mv[z + 1][y][x];
        double J[3] = {0.0, 0.0, 0.0};
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
        const long long o = (((long long) i * B.N1 + j) * B.N2 + k) * 4;
        out[o + 0] = 1. / 6 * (Mi + Mj + Mk);
        out[o + 1] = J[0];
        out[o + 2] = J[1];
        out[o + 3] = J[2];
    }
}

} // namespace mara
