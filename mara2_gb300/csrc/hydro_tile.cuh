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
//   3. per zone: divergence, the RK combine on the FP32-pair accumulator
//      (or, with ACC64, on an FP64 accumulator), store; on the last stage
//      also the zone's Courant time step.
// The state lives only as conserved densities (no primitive or flux arrays
// in HBM), so a stage moves 8 bytes per field per zone for each of: the
// stage input, U0 (stages after the first) and the output, with either
// accumulator.
#pragma once

#include "physics_fp32.cuh"

namespace mara {

struct HGrid {
    float* Uh[3];      // FP32-pair conserved densities, SoA, 5 fields (with an
    float* Ul[3];      // FP64 accumulator: Uh holds the doubles, Ul the same
                       // values rounded to FP32, which the halo staging reads)
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



// ---- the FP32 arithmetic of the fused kernels --------------------------------
// Every operation is an explicitly rounded intrinsic or a PTX approximate
// reciprocal / square root, so that no multiply and add are fused differently
// in different kernels: the stage kernels, the cluster driver loop and the
// pipelined host step give the same bits from the same state.
__device__ __forceinline__ float f_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float f_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float f_sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float f_fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ float f_rcp(float a)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(a));
    return r;
}
__device__ __forceinline__ float f_sqrt(float a)
{
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(a));
    return r;
}

// NewtonianHydro::fromConserved (ConservationLaws.cpp:292-318) in FP32
__device__ __forceinline__ void fh_cons(float gamma, const float* U, float* P)
{
    const float ir = f_rcp(U[0]);
    const float mm = f_fma(U[3], U[3], f_fma(U[2], U[2], f_mul(U[1], U[1])));
    P[0] = U[0];
    P[1] = f_mul(U[1], ir);
    P[2] = f_mul(U[2], ir);
    P[3] = f_mul(U[3], ir);
    P[4] = f_mul(f_fma(f_mul(-0.5f, mm), ir, U[4]), f_sub(gamma, 1.0f));
}

// NewtonianHydro::fromPrimitive (ConservationLaws.cpp:253-290) for the face
// normal along axis AXIS
template <int AXIS>
__device__ __forceinline__ void fh_prim(float gamma, const float* P, StateF<5>& S)
{
    const float cs = f_sqrt(f_mul(f_mul(gamma, P[4]), f_rcp(P[0])));
    const float vv = f_fma(P[3], P[3], f_fma(P[2], P[2], f_mul(P[1], P[1])));
    const float vn = P[1 + AXIS];
#pragma unroll
    for (int q = 0; q < 5; ++q) S.P[q] = P[q];
    S.U[0] = P[0];
    S.U[1] = f_mul(P[0], P[1]);
    S.U[2] = f_mul(P[0], P[2]);
    S.U[3] = f_mul(P[0], P[3]);
    S.U[4] = f_fma(f_mul(0.5f, P[0]), vv, f_mul(P[4], f_rcp(f_sub(gamma, 1.0f))));
    S.F[0] = f_mul(vn, S.U[0]);
#pragma unroll
    for (int d = 0; d < 3; ++d) S.F[1 + d] = d == AXIS ? f_fma(vn, S.U[1 + d], P[4]) : f_mul(vn, S.U[1 + d]);
    S.F[4] = f_mul(vn, f_add(S.U[4], P[4]));
    S.amax = fmaxf(f_add(vn, cs), 0.0f);
    S.amin = fminf(f_sub(vn, cs), 0.0f);
}

// HlleRiemannSolver::solve (RiemannSolvers.cpp:38-57)
__device__ __forceinline__ void fh_hlle(const StateF<5>& L, const StateF<5>& R, float* F)
{
    const float ap = fmaxf(L.amax, R.amax);
    const float am = fminf(L.amin, R.amin);
    const float id = f_rcp(f_sub(ap, am));
    const float apam = f_mul(ap, am);
#pragma unroll
    for (int q = 0; q < 5; ++q)
        F[q] = f_mul(f_fma(apam, f_sub(R.U[q], L.U[q]), f_fma(ap, L.F[q], f_mul(-am, R.F[q]))), id);
}

// the star-state flux of one side (RiemannSolvers.cpp:86-115): S the side's
// wave speed, m = rho (S - vn)
template <int AXIS>
__device__ __forceinline__ void fh_hllc_star(const StateF<5>& K, float S, float m, float lc, float* F)
{
    const float* P = K.P;
    const float vn = P[1 + AXIS];
    const float f = f_mul(m, f_rcp(f_sub(S, lc)));
    float Us[5];
    Us[0] = f;
    Us[4] = f_mul(f, f_fma(f_sub(lc, vn), f_add(lc, f_mul(P[4], f_rcp(m))), f_mul(K.U[4], f_rcp(P[0]))));
#pragma unroll
    for (int d = 0; d < 3; ++d) Us[1 + d] = d == AXIS ? f_mul(f, f_add(f_sub(lc, vn), P[1 + d])) : f_mul(f, P[1 + d]);
#pragma unroll
    for (int i = 0; i < 5; ++i) F[i] = f_fma(S, f_sub(Us[i], K.U[i]), K.F[i]);
}

// HllcNewtonianHydroRiemannSolver::solve (RiemannSolvers.cpp:63-118)
template <int AXIS>
__device__ __forceinline__ void fh_hllc(const StateF<5>& L, const StateF<5>& R, float* F)
{
    const float ap = fmaxf(L.amax, R.amax);
    const float am = fminf(L.amin, R.amin);
    const float vnl = L.P[1 + AXIS], vnr = R.P[1 + AXIS];
    const float ml = f_mul(L.P[0], f_sub(am, vnl)), mr = f_mul(R.P[0], f_sub(ap, vnr));
    const float lc = f_mul(f_sub(f_fma(-mr, vnr, R.P[4]), f_fma(-ml, vnl, L.P[4])), f_rcp(f_sub(ml, mr)));
    if (0.0f <= am) {
#pragma unroll
        for (int i = 0; i < 5; ++i) F[i] = L.F[i];
    } else if (0.0f <= lc) {
        fh_hllc_star<AXIS>(L, am, ml, lc, F);
    } else if (0.0f <= ap) {
        fh_hllc_star<AXIS>(R, ap, mr, lc, F);
    } else {
#pragma unroll
        for (int i = 0; i < 5; ++i) F[i] = R.F[i];
    }
}

// generalized minmod (Reconstruction.cpp:55-61), see minmod_f
__device__ __forceinline__ float fh_minmod(float theta, float ul, float u0, float ur)
{
    const float a = f_mul(theta, f_sub(u0, ul));
    const float b = f_mul(0.5f, f_sub(ur, ul));
    const float c = f_mul(theta, f_sub(ur, u0));
    const float m = fminf(fabsf(a), fminf(fabsf(b), fabsf(c)));
    return f_mul(a, c) > 0.0f ? copysignf(m, a) : 0.0f;
}

template <int RECON>
__device__ __forceinline__ void recon_pair(const float* v, float theta, float& L, float& R)
{
    // v[0..2G-1] straddles the face between v[G-1] and v[G]
    if constexpr (RECON == RECON_PCM) {
        L = v[0];
        R = v[1];
    } else {
        L = f_fma(0.5f, fh_minmod(theta, v[0], v[1], v[2]), v[1]);
        R = f_fma(-0.5f, fh_minmod(theta, v[1], v[2], v[3]), v[2]);
    }
}

// the flux through a face whose normal is along axis AXIS
template <int RIEMANN, int AXIS>
__device__ __forceinline__ void hydro_face_flux(float gamma, const float* PL, const float* PR, float* F)
{
    StateF<5> L, R;
    fh_prim<AXIS>(gamma, PL, L);
    fh_prim<AXIS>(gamma, PR, R);
    if constexpr (RIEMANN == RIEMANN_HLLC) fh_hllc<AXIS>(L, R, F);
    else fh_hlle(L, R, F);
}

// Courant step of one zone: lmin / max over x, y, z of max |eigenvalue|
// (FieldOperator::getCourantTimestep); for hydro max |A| = max|v_a| + cs.
__device__ __forceinline__ float hydro_zone_dt(float gamma, float lmin, const float* U)
{
    float P[5];
    fh_cons(gamma, U, P);
    const float cs = f_sqrt(f_mul(f_mul(gamma, P[4]), f_rcp(P[0])));
    const float vmax = fmaxf(fabsf(P[1]), fmaxf(fabsf(P[2]), fabsf(P[3])));
    return f_mul(lmin, f_rcp(f_add(vmax, cs)));
}

__device__ __forceinline__ float hydro_zone_dt(const HGrid& g, const float* U) { return hydro_zone_dt(g.gamma, g.lmin, U); }

// the update of one field of one zone: L = -(F+ - F-) / dx (- (G+ - G-) / dy),
// U = rk_combine(U0, U, dt L)
__device__ __forceinline__ float fh_div(float fm, float fp, float idx) { return f_mul(f_sub(fm, fp), idx); }
__device__ __forceinline__ float fh_div(float fm, float fp, float idx, float gm, float gp, float idy)
{
    return f_fma(f_sub(gm, gp), idy, fh_div(fm, fp, idx));
}

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

// The faces of a 2-D PLM tile are computed in runs: a run is RL consecutive
// faces along their normal in one row (x faces) or column (y faces), RL
// chosen so that the tile's runs about fill the block once, and a run forms
// each zone's limited slope once for the right state of the face on the
// zone's left and the left state of the face on its right: (RL + 1) / (2 RL)
// of the minmods of faces taken one at a time, with the same bits.
template <int DIM, int RECON, int TX, int TY, int NT>
struct FaceRuns {
    static constexpr bool ON = DIM == 2 && RECON == RECON_PLM;
    static constexpr int NF = (TX + 1) * TY + TX * (TY + 1);
    static constexpr int RL0 = NF / NT < 1 ? 1 : NF / NT;
    static constexpr int RL = RL0 > TY + 1 ? TY + 1 : RL0;
    static constexpr int SX = (TX + 1) / RL, SY = (TY + 1) / RL;   // runs per row / per column
    static constexpr int LX = (TX + 1) / SX, LY = (TY + 1) / SY;   // faces per run but the last
    static constexpr int NXR = SX * TY, NR = NXR + SY * TX;
    // the runs of a row (n = TX + 1 faces, S runs of L) or a column cover
    // its faces once each, in order, with no run empty
    static constexpr bool covers(int n, int S, int L)
    {
        int next = 0;
        for (int j = 0; j < S; ++j) {
            const int a = j * L, e = j == S - 1 ? n : a + L;
            if (a != next || e <= a) return false;
            next = e;
        }
        return next == n;
    }
    static constexpr bool VALID = !ON || (covers(TX + 1, SX, LX) && covers(TY + 1, SY, LY));
};

// shared memory of one tile stage; under face runs the primitives' rows
// have an odd pitch, which spreads the x runs a warp reads over the banks
// (at most 2-way conflicts for a 32 x 16 tile)
template <int DIM, int RECON, int TX, int TY>
struct TileSmem {
    static constexpr int G = HaloOf<RECON>::G;
    static constexpr int PAD = (DIM == 2 && RECON == RECON_PLM && (TX + 2 * G) % 2 == 0) ? 1 : 0;
    float Ps[5][DIM == 2 ? TY + 2 * G : 1][TX + 2 * G + PAD];
    float Uc[5][TY][TX];   // the stage input's high words of the tile's zones (EARLY or RUNS)
    float Fx[5][TY][TX + 1];
    float Fy[5][DIM == 2 ? TY + 1 : 1][DIM == 2 ? TX : 1];
};

// PLM fluxes of the faces a .. e-1 of row `line` (AXIS 0: x faces, face f
// left of tile zone f) or column `line` (AXIS 1: y faces, face f below tile
// row f) of a tile, in order.  Each zone's limited slope s is formed once:
// fma(-1/2, s, u) is the right state of the face on the zone's left and
// fma(1/2, s, u) the left state of the face on its right, the values
// recon_pair forms one face at a time.
template <int RIEMANN, int AXIS, int DIM, int RECON, int TX, int TY>
__device__ __forceinline__ void plm_face_run(TileSmem<DIM, RECON, TX, TY>& sm, int line, int a, int e, float theta,
                                             float gamma)
{
    constexpr int G = HaloOf<RECON>::G;
    // primitive k of the line's stencil (k = f + 1 and f + 2 straddle face f)
    auto ps = [&](int q, int k) -> float { return AXIS == 0 ? sm.Ps[q][line + G][k] : sm.Ps[q][k][line + G]; };
    float u1[5], u2[5], PL[5];
#pragma unroll
    for (int q = 0; q < 5; ++q) {
        const float u0 = ps(q, a);
        u1[q] = ps(q, a + 1);
        u2[q] = ps(q, a + 2);
        PL[q] = f_fma(0.5f, fh_minmod(theta, u0, u1[q], u2[q]), u1[q]);
    }
#pragma unroll 1
    for (int f = a; f < e; ++f) {
        float PR[5], NL[5], Fh[5];
#pragma unroll
        for (int q = 0; q < 5; ++q) {
            const float u3 = ps(q, f + 3);
            const float s = fh_minmod(theta, u1[q], u2[q], u3);
            PR[q] = f_fma(-0.5f, s, u2[q]);
            NL[q] = f_fma(0.5f, s, u2[q]);
            u1[q] = u2[q];
            u2[q] = u3;
        }
        hydro_face_flux<RIEMANN, AXIS>(gamma, PL, PR, Fh);
#pragma unroll
        for (int q = 0; q < 5; ++q) {
            if (AXIS == 0) sm.Fx[q][line][f] = Fh[q];
            else sm.Fy[q][f][line] = Fh[q];
            PL[q] = NL[q];
        }
    }
}

// a load of the state: through L1 in the stage kernels (nothing a stage
// reads changes during its launch), from L2 where CTAs of one launch read
// what other CTAs of it wrote
template <bool L2ONLY>
__device__ __forceinline__ float ld_state(const float* p)
{
    if constexpr (L2ONLY) return __ldcg(p);
    else return *p;
}

// RK weight b of SolutionSchemes.cpp:135-138 in FP64 from its FP32 form
// (1, 1/2, 1/4 or 2/3)
__device__ __forceinline__ double rk_b_fp64(float b)
{
    return b == 1.0f ? 1.0 : b == 0.5f ? 0.5 : b == 0.25f ? 0.25 : 2.0 / 3.0;
}

// U_new = U0 (1 - b) + (U + dt L) b (SolutionSchemes.cpp:232-235) on the FP64
// accumulator; dt L is the FP32 flux arithmetic's product, exact in FP64
__device__ __forceinline__ double rk_combine_d(double U0, double U, float dtL, float b)
{
    const double s = __dadd_rn(U, f2d_exact(dtL));
    if (b == 1.0f) return s;
    if (b == 0.5f) return half_exact(__dadd_rn(U0, s));
    const double bd = rk_b_fp64(b);
    return __dadd_rn(__dmul_rn(U0, __dsub_rn(1.0, bd)), __dmul_rn(s, bd));
}

// One RK stage of one tile of grid g whose state is in rotation buffer s:
//   src: buffer holding the stage input; dst: buffer written; buffer s
//   holds U0 (read per zone); b, omb = b, 1 - b; on the last stage the
//   tile's Courant step goes to *at.cfl().  at.dt() and at.cfl() are read
//   where they are used, so that neither holds registers across the tile;
//   at.proceed() (the same in every thread of the CTA) is asked before the
//   update: false leaves the tile's state as it was.
//   ACC64: the state arrays Uh hold the FP64 accumulator, Ul its FP32 copy.
//   EARLY: the FP32-pair update's operands loaded before the barrier that
//   ends the face phase (registers for 3 CTAs of 256 threads per SM).
//   RUNS: a 2-D PLM tile's faces in runs (FaceRuns), else one face per
//   thread at a time; and the tile's stage-input high words kept in shared
//   memory by the staging for the update.
template <int DIM, int RECON, int RIEMANN, int TX, int TY, int NT, bool L2ONLY, bool ACC64 = false, bool EARLY = false,
          bool RUNS = false,
          class At>
__device__ __forceinline__ void tile_stage(TileSmem<DIM, RECON, TX, TY>& sm, const HGrid& g, const TileRef& tr,
                                           int s, int stage, float b, float omb, int last, const At& at)
{
    constexpr int G = HaloOf<RECON>::G;
    constexpr int WX = TX + 2 * G;
    constexpr int WY = DIM == 2 ? TY + 2 * G : 1;
    constexpr int FXN = (TX + 1) * TY;
    constexpr int FYN = DIM == 2 ? TX * (TY + 1) : 1;
    // buffer rotation: stage input / output per RK stage
    int src, dst;
    if (stage == 0) { src = s; dst = last ? (s ^ 1) : (s + 1) % 3; }
    else if (stage == 1) { src = (s + 1) % 3; dst = last ? s : (s + 2) % 3; }
    else { src = (s + 2) % 3; dst = s; }
    // the stage input's FP32 values: the pairs' high words, or the FP64
    // accumulator's FP32 copy
    const float* __restrict__ Uin = ACC64 ? g.Ul[src] : g.Uh[src];
    const long long sU = g.sU;
    const int n0 = g.n0, n1 = g.n1;

    // L2 prefetch of what the update phase reads per zone besides the
    // stage input's FP32 values (staged below): the pairs' low words and,
    // after the first stage, both words of U0; or the FP64 accumulators of
    // the stage input and, after the first stage, of U0
    {
        const int rows = DIM == 2 ? TY : 1;
        constexpr int W = ACC64 ? 8 : 4;                 // bytes per element
        const int per = (TX * W + 127) / 128;            // 128-byte lines per row segment
        const int arrays = ACC64 ? (stage == 0 ? 1 : 2) : (stage == 0 ? 1 : 3);
        const int lines = arrays * 5 * rows * per;
        for (int l = threadIdx.x; l < lines; l += NT) {
            const int seg = l % per, r = (l / per) % rows, q = (l / (per * rows)) % 5, a = l / (per * rows * 5);
            const int y = tr.y0 + r, x = tr.x0 + seg * (128 / W);
            if (y < n1 && x < n0) {
                const float* base = ACC64 ? (a == 0 ? g.Uh[src] : g.Uh[s])
                                          : a == 0 ? g.Ul[src] : a == 1 ? g.Uh[s] : g.Ul[s];
                const char* ptr = reinterpret_cast<const char*>(base) + ((long long) q * sU + (long long) y * n0 + x) * W;
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
            const long long base = (long long) (tr.y0 - (DIM == 2 ? G : 0)) * n0 + (tr.x0 - G);
#pragma unroll
            for (int k = 0; k < NC; ++k) {
                const int c = threadIdx.x + k * NT;
                fl[k] = 0;
                if (c < WX * WY) {
                    const int lx = c % WX, ly = c / WX;
                    const long long p = base + (long long) ly * n0 + lx;
#pragma unroll
                    for (int q = 0; q < 5; ++q) Ur[k][q] = ld_state<L2ONLY>(Uin + p + q * sU);
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
                    for (int q = 0; q < 5; ++q) Ur[k][q] = ld_state<L2ONLY>(Uin + q * sU + o);
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
                if constexpr ((EARLY || RUNS) && !ACC64) {
                    // a zone of the tile itself: keep its conserved high words
                    // for the update (halo zones of a tile never are)
                    const int zx = lx - G, zy = DIM == 2 ? ly - G : 0;
                    if (zx >= 0 && zx < TX && zy >= 0 && zy < TY) {
#pragma unroll
                        for (int q = 0; q < 5; ++q) sm.Uc[q][zy][zx] = Ur[k][q];
                    }
                }
                float P[5];
                fh_cons(g.gamma, Ur[k], P);
#pragma unroll
                for (int q = 0; q < 5; ++q) sm.Ps[q][ly][lx] = P[q];
            }
        }
    }
    __syncthreads();

    const float theta = g.plm_theta, gamma = g.gamma;
    // 2. x faces and y faces (face fx sits left of tile zone fx, face fy
    //    below tile row fy): in runs along their normals (2-D PLM), else one
    //    face per thread in one balanced loop
    using Runs = FaceRuns<DIM, RECON, TX, TY, NT>;
    static_assert(Runs::VALID, "face runs must cover every face of a tile line once");
    if constexpr (RUNS && Runs::ON) {
        for (int r = threadIdx.x; r < Runs::NR; r += NT) {
            if (r < Runs::NXR) {
                // the runs of one index in every row side by side, so that the
                // longer last runs of the rows share warps (a 32 x 16 tile: 17
                // warp iterations over the x faces instead of 20)
                const int j = r / TY, fy = r % TY;
                const int a = j * Runs::LX, e = j == Runs::SX - 1 ? TX + 1 : a + Runs::LX;
                plm_face_run<RIEMANN, 0>(sm, fy, a, e, theta, gamma);
            } else {
                const int h = r - Runs::NXR;
                const int fx = h % TX, j = h / TX;
                const int a = j * Runs::LY, e = j == Runs::SY - 1 ? TY + 1 : a + Runs::LY;
                plm_face_run<RIEMANN, 1>(sm, fx, a, e, theta, gamma);
            }
        }
    } else
    for (int f = threadIdx.x; f < FXN + (DIM == 2 ? FYN : 0); f += NT) {
        float PL[5], PR[5], Fh[5];
        if (f < FXN) {
            const int fx = f % (TX + 1), fy = f / (TX + 1);
            const int ry = DIM == 2 ? fy + G : 0;
#pragma unroll
            for (int q = 0; q < 5; ++q) {
                float v[2 * G];
#pragma unroll
                for (int m = 0; m < 2 * G; ++m) v[m] = sm.Ps[q][ry][fx + m];
                recon_pair<RECON>(v, theta, PL[q], PR[q]);
            }
            hydro_face_flux<RIEMANN, 0>(gamma, PL, PR, Fh);
#pragma unroll
            for (int q = 0; q < 5; ++q) sm.Fx[q][fy][fx] = Fh[q];
        } else if constexpr (DIM == 2) {
            const int h = f - FXN;
            const int fx = h % TX, fy = h / TX;
#pragma unroll
            for (int q = 0; q < 5; ++q) {
                float v[2 * G];
#pragma unroll
                for (int m = 0; m < 2 * G; ++m) v[m] = sm.Ps[q][fy + m][fx + G];
                recon_pair<RECON>(v, theta, PL[q], PR[q]);
            }
            hydro_face_flux<RIEMANN, 1>(gamma, PL, PR, Fh);
#pragma unroll
            for (int q = 0; q < 5; ++q) sm.Fy[q][fy][fx] = Fh[q];
        }
    }

    // 3. divergence, RK combine, store.  The stage input and output are
    // distinct buffers; an RK2 last stage writes U0's own buffer, where each
    // element is read before the value computed from it is written.
    const float* __restrict__ U0h = g.Uh[s];
    const float* __restrict__ U0l = g.Ul[s];
    const float* __restrict__ Uph = g.Uh[src];
    const float* __restrict__ Upl = g.Ul[src];
    float* __restrict__ Unh = g.Uh[dst];
    float* __restrict__ Unl = g.Ul[dst];
    const float idx = g.idx, idy = g.idy;
    float zdt = 3.0e38f;
    if constexpr (EARLY && !ACC64) {
        // Each thread's zones' operands from HBM (the stage input's low
        // words and, after the first stage, both words of U0; the high words
        // of the stage input were kept in shared memory when the tile was
        // staged) are loaded before the barrier that ends the face phase, so
        // that their latency overlaps the wait for the other threads' faces.
        // Nothing in this launch writes them before this CTA's own stores.
        constexpr int NZ = (TX * TY + NT - 1) / NT;
        float r_pl[NZ][5], r_0h[NZ][5], r_0l[NZ][5];
        auto load = [&](int z) {
            const int c = threadIdx.x + z * NT;
            const int x = tr.x0 + c % TX, y = tr.y0 + c / TX;
            if (c < TX * TY && x < n0 && y < n1) {
                const long long o = (long long) y * n0 + x;
#pragma unroll
                for (int q = 0; q < 5; ++q) {
                    r_pl[z][q] = ld_state<L2ONLY>(Upl + q * sU + o);
                    // U0 enters only with b < 1 (stage 1 is U + dt L)
                    r_0h[z][q] = b == 1.0f ? 0.0f : ld_state<L2ONLY>(U0h + q * sU + o);
                    r_0l[z][q] = b == 1.0f ? 0.0f : ld_state<L2ONLY>(U0l + q * sU + o);
                }
            }
        };
#pragma unroll
        for (int z = 0; z < NZ; ++z) load(z);
        __syncthreads();
        if (!at.proceed()) return;
        const float dt = at.dt();
#pragma unroll
        for (int z = 0; z < NZ; ++z) {
            const int c = threadIdx.x + z * NT;
            const int lx = c % TX, ly = c / TX;
            const int x = tr.x0 + lx, y = tr.y0 + ly;
            if (c >= TX * TY || x >= n0 || y >= n1) continue;
            const long long o = (long long) y * n0 + x;
            float Unew[5];
#pragma unroll
            for (int q = 0; q < 5; ++q) {
                float L;
                if constexpr (DIM == 2)
                    L = fh_div(sm.Fx[q][ly][lx], sm.Fx[q][ly][lx + 1], idx, sm.Fy[q][ly][lx], sm.Fy[q][ly + 1][lx], idy);
                else
                    L = fh_div(sm.Fx[q][ly][lx], sm.Fx[q][ly][lx + 1], idx);
                const df Un = rk_combine(df{r_0h[z][q], r_0l[z][q]}, df{sm.Uc[q][ly][lx], r_pl[z][q]}, f_mul(dt, L), b, omb);
                Unh[q * sU + o] = Un.hi;
                Unl[q * sU + o] = Un.lo;
                Unew[q] = Un.hi;
            }
            if (last) zdt = fminf(zdt, hydro_zone_dt(g, Unew));
        }
    } else {
        // operands loaded zone by zone after the barrier (the kernels that
        // run a tile stage inside a larger loop keep to 64 registers)
        __syncthreads();
        if (!at.proceed()) return;
        const float dt = at.dt();
        for (int c = threadIdx.x; c < TX * TY; c += NT) {
            const int lx = c % TX, ly = c / TX;
            const int x = tr.x0 + lx, y = tr.y0 + ly;
            if (x >= n0 || y >= n1) continue;
            const long long o = (long long) y * n0 + x;
            float Unew[5];
#pragma unroll
            for (int q = 0; q < 5; ++q) {
                float L;
                if constexpr (DIM == 2)
                    L = fh_div(sm.Fx[q][ly][lx], sm.Fx[q][ly][lx + 1], idx, sm.Fy[q][ly][lx], sm.Fy[q][ly + 1][lx], idy);
                else
                    L = fh_div(sm.Fx[q][ly][lx], sm.Fx[q][ly][lx + 1], idx);
                if constexpr (ACC64) {
                    const double* U0d = reinterpret_cast<const double*>(U0h) + q * sU + o;
                    const double* Upd = reinterpret_cast<const double*>(Uph) + q * sU + o;
                    const double u0 = b == 1.0f ? 0.0 : (L2ONLY ? __ldcg(U0d) : *U0d);
                    const double Un = rk_combine_d(u0, L2ONLY ? __ldcg(Upd) : *Upd, f_mul(dt, L), b);
                    reinterpret_cast<double*>(Unh)[q * sU + o] = Un;
                    Unew[q] = d2f_rn_ftz(Un);
                    Unl[q * sU + o] = Unew[q];   // the FP32 copy the next stage stages
                } else {
                    // U0 enters only with b < 1 (stage 1 is U + dt L)
                    const df U0 = b == 1.0f ? df{0.0f, 0.0f}
                                            : df{ld_state<L2ONLY>(U0h + q * sU + o), ld_state<L2ONLY>(U0l + q * sU + o)};
                    // the stage input's high words: kept in shared memory by the
                    // staging under face runs
                    const df Up = {RUNS ? sm.Uc[q][ly][lx] : ld_state<L2ONLY>(Uph + q * sU + o),
                                   ld_state<L2ONLY>(Upl + q * sU + o)};
                    const df Un = rk_combine(U0, Up, f_mul(dt, L), b, omb);
                    Unh[q * sU + o] = Un.hi;
                    Unl[q * sU + o] = Un.lo;
                    Unew[q] = Un.hi;
                }
            }
            if (last) zdt = fminf(zdt, hydro_zone_dt(g, Unew));
        }
    }
    if (last) block_min_to(at.cfl(), zdt);
}

// The stage kernel's form for a tile shape: 2-D PLM tiles take their faces
// in runs at 4 CTAs of 256 threads per SM (64 registers a thread, no
// spills; KH 1024^2 with FP32 pairs 0.0880 ms a step against 0.0957 ms at 3
// CTAs and 0.0903 ms for one face per thread with the early operand loads).
// The other FP32-pair tiles keep one face per thread with the early loads at
// 3 CTAs (80 registers), 11 % faster than 4 CTAs without them on 1-D tiles
// of 256 zones; the FP64-accumulator form has no early loads and runs at 4
// CTAs.  ONEFACE keeps a 2-D PLM tile at one face per thread with the
// early loads (the batch's 32 x 16 tiles on small grids, where it measured
// faster).
template <int DIM, int RECON, int TX, int TY, int NT, bool ACC64, bool ONEFACE = false> struct TileForm {
    static constexpr bool RUNS = FaceRuns<DIM, RECON, TX, TY, NT>::ON && !ONEFACE;
    static constexpr bool EARLY = !RUNS && !ACC64;
    static constexpr int CTAS = EARLY ? 768 / NT : 1024 / NT;
};

// One RK stage over a list of tiles (persistent: CTAs stride over tiles).
template <int DIM, int RECON, int RIEMANN, int TX, int TY, int NT, bool ACC64 = false, bool ONEFACE = false>
__global__ void __launch_bounds__(NT, (TileForm<DIM, RECON, TX, TY, NT, ACC64, ONEFACE>::CTAS))
    hydro_tile_kernel(const HGrid* __restrict__ grids, const TileRef* __restrict__ tiles,
                      const int* __restrict__ ntiles_p,
                      const int* __restrict__ rot,  // per grid: state buffer s
                      const double* __restrict__ dtg, int dt_stride, const int* __restrict__ done, int done_stride,
                      int stage, float b, float omb, int last, unsigned long long* __restrict__ cfl, int cfl_stride,
                      int after_begin)
{
    __shared__ TileSmem<DIM, RECON, TX, TY> sm;
    const int ntiles = *ntiles_p;  // device-resident so a captured graph follows a changing tile list
    // after_begin: launched as the programmatic dependent of the step-start
    // kernel (dt, done, the Courant slot's reset), so the tile staging and
    // the faces, which need none of these, overlap it; the update waits for
    // it and reads whether the step is taken.  Otherwise a finished grid's
    // tiles are skipped whole.
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const TileRef tr = tiles[t];
        const HGrid& g = grids[tr.grid];
        if (!after_begin && done[tr.grid * done_stride]) continue;
        struct {
            const double* dtp;
            unsigned long long* slot;
            const int* donep;
            int wait;
            __device__ float dt() const { return (float) *dtp; }
            __device__ unsigned long long* cfl() const { return slot; }
            __device__ bool proceed() const
            {
                if (!wait) return true;
                asm volatile("griddepcontrol.wait;" ::: "memory");
                return *(volatile const int*) donep == 0;
            }
        } at{dtg + tr.grid * dt_stride, cfl + tr.grid * cfl_stride, done + tr.grid * done_stride, after_begin};
        using Form = TileForm<DIM, RECON, TX, TY, NT, ACC64, ONEFACE>;
        tile_stage<DIM, RECON, RIEMANN, TX, TY, NT, false, ACC64, Form::EARLY, Form::RUNS>(sm, g, tr, rot[tr.grid], stage, b,
                                                                                    omb, last, at);
    }
}

} // namespace mara
