// hydro_tile.cuh -- fused RK-stage kernel for Newtonian hydro on 1-D and 2-D
// Cartesian grids, mixed precision, shared by the single-grid mixed path
// (mixed.cu) and the batched / serving path (batch.cu).
//
// One CTA owns a TX x TY tile of interior zones and does a whole RK stage
// of MethodOfLinesTVD::advance (SolutionSchemes.cpp:191-274) for it:
//   1. stage the tile plus a stencil-wide halo of conserved densities (FP32
//      high word) in shared memory as primitives (fromConserved); halo zones
//      outside the grid come from the boundary condition's interior image
//      (periodic wrap, outflow clamp, reflecting mirror with the normal
//      momentum negated), axis by axis as applySimple composes them;
//   2. x-face fluxes, then y-face fluxes (reconstruction + fromPrimitive x2
//      + Riemann solver) into shared memory;
//   3. per zone: divergence, the RK combine on the FP32-pair accumulator,
//      store; on the last stage also the zone's Courant time step.
// The state lives only as conserved densities (no primitive or flux arrays
// in HBM), so a stage moves 8 bytes per field per zone for each of: the
// stage input, U0 (stages after the first) and the output.
#pragma once

#include "physics_fp32.cuh"

namespace mara {

struct HGrid {
    float* Uh[3];      // FP32-pair conserved densities, SoA, 5 fields
    float* Ul[3];
    long long sU;      // field stride (n0 * n1)
    int n0, n1;        // interior zones (n1 = 1 for 1-D)
    int bc;
    float gamma;
    float plm_theta;
    float idx, idy;    // 1/dx, 1/dy
    float lmin;        // MeshOperator::linearCellDimension
};

struct TileRef {
    int grid;
    int x0, y0;
    int pad;
};

// boundary image of interior coordinate x on an axis of n zones; flips the
// momentum component when the image is a reflection
__device__ __forceinline__ int bc_image(int x, int n, int bc, int& flip)
{
    if (x >= 0 && x < n) return x;
    if (bc == BC_PERIODIC) {
        x %= n;
        if (x < 0) x += n;
    } else if (bc == BC_OUTFLOW) {
        x = x < 0 ? 0 : n - 1;
    } else {
        flip ^= 1;
        x = x < 0 ? -1 - x : 2 * n - 1 - x;
    }
    return x < 0 ? 0 : (x >= n ? n - 1 : x);
}

// Hydro primitive <-> conserved conversion in double precision at the host
// boundary of the mixed-precision forms.  Every operation is rounded on its
// own (no multiply-add contraction), so the single-grid and the batched
// loaders and stores produce the same bits from the same primitives.
__device__ __forceinline__ void hydro_p2u_d(const double* P, double inv_gm1, double* U)
{
    const double vv = __dadd_rn(__dadd_rn(__dmul_rn(P[1], P[1]), __dmul_rn(P[2], P[2])), __dmul_rn(P[3], P[3]));
    U[0] = P[0];
    U[1] = __dmul_rn(P[0], P[1]);
    U[2] = __dmul_rn(P[0], P[2]);
    U[3] = __dmul_rn(P[0], P[3]);
    U[4] = __dadd_rn(__dmul_rn(__dmul_rn(0.5, P[0]), vv), __dmul_rn(P[4], inv_gm1));
}

__device__ __forceinline__ void hydro_u2p_d(const double* U, double gm1, double* P)
{
    const double ir = 1.0 / U[0];
    const double pp = __dadd_rn(__dadd_rn(__dmul_rn(U[1], U[1]), __dmul_rn(U[2], U[2])), __dmul_rn(U[3], U[3]));
    P[0] = U[0];
    P[1] = __dmul_rn(U[1], ir);
    P[2] = __dmul_rn(U[2], ir);
    P[3] = __dmul_rn(U[3], ir);
    P[4] = __dmul_rn(__dsub_rn(U[4], __dmul_rn(__dmul_rn(0.5, pp), ir)), gm1);
}

template <int RECON> struct HaloOf { static constexpr int G = RECON == RECON_PCM ? 1 : 2; };

template <int RECON>
__device__ __forceinline__ void recon_pair(const float* v, float theta, float& L, float& R)
{
    // v[0..2G-1] straddles the face between v[G-1] and v[G]
    if constexpr (RECON == RECON_PCM) {
        L = v[0];
        R = v[1];
    } else {
        L = v[1] + 0.5f * minmod_f(theta, v[0], v[1], v[2]);
        R = v[2] - 0.5f * minmod_f(theta, v[1], v[2], v[3]);
    }
}

template <int RIEMANN>
__device__ __forceinline__ void hydro_face_flux(float gamma, const float* PL, const float* PR, const float* n, float* F)
{
    StateF<5> L, R;
    hydro_prim_f(gamma, PL, n, L);
    hydro_prim_f(gamma, PR, n, R);
    if constexpr (RIEMANN == RIEMANN_HLLC) hllc_f<5>(L, R, n, F);
    else hlle_f<5>(L, R, F);
}

// Courant step of one zone: lmin / max over x, y, z of max |eigenvalue|
// (FieldOperator::getCourantTimestep); for hydro max |A| = max|v_a| + cs.
__device__ __forceinline__ float hydro_zone_dt(float gamma, float lmin, const float* U)
{
    float P[5];
    hydro_cons_f(gamma, U, P);
    const float cs = sqrtf(gamma * P[4] / P[0]);
    const float vmax = fmaxf(fabsf(P[1]), fmaxf(fabsf(P[2]), fabsf(P[3])));
    return lmin / (vmax + cs);
}

__device__ __forceinline__ float hydro_zone_dt(const HGrid& g, const float* U) { return hydro_zone_dt(g.gamma, g.lmin, U); }

__device__ __forceinline__ void block_min_to(unsigned long long* dst, float v)
{
    unsigned long long b = ~0ull;
    if (v > 0.f && v < 3.0e38f) b = (unsigned long long) __double_as_longlong((double) v);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const unsigned long long o = __shfl_down_sync(0xffffffffu, b, off);
        b = o < b ? o : b;
    }
    if ((threadIdx.x & 31) == 0 && b != ~0ull) atomicMin(dst, b);
}

// One RK stage over a list of tiles (persistent: CTAs stride over tiles).
//   src: buffer holding the stage input; dst: buffer written; buffer 0 of a
//   grid's rotation holds U0 (read per zone); b, omb = b, 1 - b.
template <int DIM, int RECON, int RIEMANN, int TX, int TY, int NT>
__global__ void __launch_bounds__(NT) hydro_tile_kernel(const HGrid* __restrict__ grids,
                                                        const TileRef* __restrict__ tiles,
                                                        const int* __restrict__ ntiles_p,
                                                        const int* __restrict__ rot,  // per grid: state buffer s
                                                        const double* __restrict__ dtg, int dt_stride,
                                                        const int* __restrict__ done, int done_stride,
                                                        int stage, float b, float omb, int last,
                                                        unsigned long long* __restrict__ cfl, int cfl_stride)
{
    constexpr int G = HaloOf<RECON>::G;
    constexpr int WX = TX + 2 * G;
    constexpr int WY = DIM == 2 ? TY + 2 * G : 1;
    constexpr int FXN = (TX + 1) * TY;
    constexpr int FYN = DIM == 2 ? TX * (TY + 1) : 1;
    __shared__ float Ps[5][WY][WX];
    __shared__ float Fx[5][TY][TX + 1];
    __shared__ float Fy[5][DIM == 2 ? TY + 1 : 1][TX];

    const int ntiles = *ntiles_p;  // device-resident so a captured graph follows a changing tile list
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const TileRef tr = tiles[t];
        const HGrid& g = grids[tr.grid];
        if (done[tr.grid * done_stride]) continue;
        const int s = rot[tr.grid];
        // buffer rotation: stage input / output per RK stage
        int src, dst;
        if (stage == 0) { src = s; dst = last ? (s ^ 1) : (s + 1) % 3; }
        else if (stage == 1) { src = (s + 1) % 3; dst = last ? s : (s + 2) % 3; }
        else { src = (s + 2) % 3; dst = s; }
        const float* __restrict__ Uin = g.Uh[src];
        const long long sU = g.sU;
        const int n0 = g.n0, n1 = g.n1;

        // L2 prefetch of what the update phase reads per zone besides the
        // stage input's high word (already staged below): its low word and,
        // after the first stage, both words of U0
        {
            const int rows = DIM == 2 ? TY : 1;
            const int per = (TX * 4 + 127) / 128;            // 128-byte lines per row segment
            const int arrays = stage == 0 ? 1 : 3;
            const int lines = arrays * 5 * rows * per;
            for (int l = threadIdx.x; l < lines; l += NT) {
                const int seg = l % per, r = (l / per) % rows, q = (l / (per * rows)) % 5, a = l / (per * rows * 5);
                const int y = tr.y0 + r, x = tr.x0 + seg * 32;
                if (y < n1 && x < n0) {
                    const float* base = a == 0 ? g.Ul[src] : a == 1 ? g.Uh[s] : g.Ul[s];
                    const float* ptr = base + q * sU + (long long) y * n0 + x;
                    asm volatile("prefetch.global.L2 [%0];" ::"l"(ptr));
                }
            }
        }

        __syncthreads(); // the previous tile's shared data is consumed
        // 1. primitives of the tile and its halo: all loads first, then the
        //    conversions, so each thread keeps NC x 5 loads in flight.  A tile
        //    whose halo lies inside the grid reads it as one rectangle; the
        //    others take every halo zone from its boundary image.
        {
            constexpr int NC = (WX * WY + NT - 1) / NT;
            float Ur[NC][5];
            int fl[NC];
            const bool inner = tr.x0 - G >= 0 && tr.x0 + TX + G <= n0 &&
                               (DIM == 1 || (tr.y0 - G >= 0 && tr.y0 + TY + G <= n1));
            if (inner) {
                const float* base = Uin + (long long) (tr.y0 - (DIM == 2 ? G : 0)) * n0 + (tr.x0 - G);
#pragma unroll
                for (int k = 0; k < NC; ++k) {
                    const int c = threadIdx.x + k * NT;
                    fl[k] = 0;
                    if (c < WX * WY) {
                        const int lx = c % WX, ly = c / WX;
                        const float* p = base + (long long) ly * n0 + lx;
#pragma unroll
                        for (int q = 0; q < 5; ++q) Ur[k][q] = p[q * sU];
                    }
                }
            } else {
#pragma unroll
                for (int k = 0; k < NC; ++k) {
                    const int c = threadIdx.x + k * NT;
                    fl[k] = 0;
                    if (c < WX * WY) {
                        const int lx = c % WX, ly = c / WX;
                        int flipx = 0, flipy = 0;
                        const int x = bc_image(tr.x0 + lx - G, n0, g.bc, flipx);
                        const int y = DIM == 2 ? bc_image(tr.y0 + ly - G, n1, g.bc, flipy) : 0;
                        const long long o = (long long) y * n0 + x;
#pragma unroll
                        for (int q = 0; q < 5; ++q) Ur[k][q] = Uin[q * sU + o];
                        fl[k] = flipx | (flipy << 1);
                    }
                }
            }
#pragma unroll
            for (int k = 0; k < NC; ++k) {
                const int c = threadIdx.x + k * NT;
                if (c < WX * WY) {
                    const int lx = c % WX, ly = c / WX;
                    if (fl[k] & 1) Ur[k][1] = -Ur[k][1];
                    if (fl[k] & 2) Ur[k][2] = -Ur[k][2];
                    float P[5];
                    hydro_cons_f(g.gamma, Ur[k], P);
#pragma unroll
                    for (int q = 0; q < 5; ++q) Ps[q][ly][lx] = P[q];
                }
            }
        }
        __syncthreads();

        const float theta = g.plm_theta, gamma = g.gamma;
        // 2. x faces and y faces in one balanced loop (face fx sits left of
        //    tile zone fx, face fy below tile row fy)
        for (int f = threadIdx.x; f < FXN + (DIM == 2 ? FYN : 0); f += NT) {
            float PL[5], PR[5], Fh[5];
            if (f < FXN) {
                const int fx = f % (TX + 1), fy = f / (TX + 1);
                const int ry = DIM == 2 ? fy + G : 0;
#pragma unroll
                for (int q = 0; q < 5; ++q) {
                    float v[2 * G];
#pragma unroll
                    for (int m = 0; m < 2 * G; ++m) v[m] = Ps[q][ry][fx + m];
                    recon_pair<RECON>(v, theta, PL[q], PR[q]);
                }
                const float nx[3] = {1.f, 0.f, 0.f};
                hydro_face_flux<RIEMANN>(gamma, PL, PR, nx, Fh);
#pragma unroll
                for (int q = 0; q < 5; ++q) Fx[q][fy][fx] = Fh[q];
            } else if constexpr (DIM == 2) {
                const int h = f - FXN;
                const int fx = h % TX, fy = h / TX;
#pragma unroll
                for (int q = 0; q < 5; ++q) {
                    float v[2 * G];
#pragma unroll
                    for (int m = 0; m < 2 * G; ++m) v[m] = Ps[q][fy + m][fx + G];
                    recon_pair<RECON>(v, theta, PL[q], PR[q]);
                }
                const float ny[3] = {0.f, 1.f, 0.f};
                hydro_face_flux<RIEMANN>(gamma, PL, PR, ny, Fh);
#pragma unroll
                for (int q = 0; q < 5; ++q) Fy[q][fy][fx] = Fh[q];
            }
        }
        __syncthreads();

        // 3. divergence, RK combine, store
        const float dt = (float) dtg[tr.grid * dt_stride];
        float zdt = 3.0e38f;
        // the rotation's three buffers are distinct arrays
        const float* __restrict__ U0h = g.Uh[s];
        const float* __restrict__ U0l = g.Ul[s];
        const float* __restrict__ Uph = g.Uh[src];
        const float* __restrict__ Upl = g.Ul[src];
        float* __restrict__ Unh = g.Uh[dst];
        float* __restrict__ Unl = g.Ul[dst];
        const float idx = g.idx, idy = g.idy;
        for (int c = threadIdx.x; c < TX * TY; c += NT) {
            const int lx = c % TX, ly = c / TX;
            const int x = tr.x0 + lx, y = tr.y0 + ly;
            if (x >= n0 || y >= n1) continue;
            const long long o = (long long) y * n0 + x;
            float Unew[5];
#pragma unroll
            for (int q = 0; q < 5; ++q) {
                float L = -(Fx[q][ly][lx + 1] - Fx[q][ly][lx]) * idx;
                if constexpr (DIM == 2) L -= (Fy[q][ly + 1][lx] - Fy[q][ly][lx]) * idy;
                const df U0 = {U0h[q * sU + o], U0l[q * sU + o]};
                const df Up = {Uph[q * sU + o], Upl[q * sU + o]};
                const df Un = rk_combine(U0, Up, dt * L, b, omb);
                Unh[q * sU + o] = Un.hi;
                Unl[q * sU + o] = Un.lo;
                Unew[q] = Un.hi;
            }
            if (last) zdt = fminf(zdt, hydro_zone_dt(g, Unew));
        }
        if (last) block_min_to(&cfl[tr.grid * cfl_stride], zdt);
    }
}

} // namespace mara
