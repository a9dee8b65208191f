// mixed.cu -- the mixed-precision path of one grid.
//
// State: conserved densities as FP32 pairs (hi + lo), SoA over the interior,
// in a rotation of three buffers (see hydro_tile.cuh).  Two kernel families:
//
//  * fused tiles (hydro_tile.cuh) for Newtonian hydro on 1-D / 2-D grids:
//    one kernel per RK stage, primitives and fluxes in shared memory only;
//  * the general form for every law / reconstruction / dimension: one FP32
//    face-flux kernel per axis (FP32 fluxes in HBM), then an update kernel
//    doing FP32 flux CT, divergence, the FP32-pair RK combine and the
//    primitive recovery (FP32 for hydro and MHD, FP64 Newton for RMHD), and
//    writing FP32 primitives with their guard images for the next sweep.
#include <algorithm>
#include <type_traits>
#include <cfloat>
#include <cstring>
#include <vector>

#include "diagnostics.cuh"
#include "hydro_cluster.cuh"
#include "hydro_tile.cuh"
#include "mixed.h"
#include "physics_fp32.cuh"

namespace mara {

// ---------------------------------------------------------------------------
// general form
struct GridF {
    int n[3], g[3], N[3];
    long long sP, sU, sF;
    float nrm[3][3];
    float idx[3];      // 1/dx per axis
    float lmin;
    int bc, ct;
    float gamma, plm_theta, shenzha_A, pressure_floor;
    int weno_is;
    double gamma_d, pfloor_d;
    double gm1_d, inv_gm1_d;
    float rm_gamf_hi, rm_gamf_lo;  // (gamma - 1) / gamma as an FP32 pair
    float rm_hcoef;                // gamma / (gamma - 1)
};

template <int RECON> struct SOf { static constexpr int S = RECON == RECON_PCM ? 1 : RECON == RECON_PLM ? 2 : 3; };

// The face fluxes along one axis of the general form.  AXIS >= 0 is the
// axis at compile time (no multiplications by the zero components of the
// normal); AXIS < 0 takes it, and the normal, at run time.
// The general form's kernels run as a chain of programmatic dependent
// launches: each waits for the kernel before it (whose writes are then
// visible) and then lets the next one launch, so a launch's start overlaps
// its predecessor's last wave.  Outside such a chain both are no-ops.
__device__ __forceinline__ void pdl_chain()
{
    asm volatile("griddepcontrol.wait;\n\tgriddepcontrol.launch_dependents;" ::: "memory");
}

template <int LAW, int RECON, int RIEMANN, int AXIS>
__global__ void __launch_bounds__(128) flux_f_kernel(const float* __restrict__ P, float* __restrict__ F, GridF G,
                                                     int axis, int lo0, int lo1, int lo2, int nb0, int nb1,
                                                     const int* __restrict__ done, DevStatus* st)
{
    pdl_chain();
    if constexpr (AXIS >= 0) axis = AXIS;
    constexpr int NQ = LawInfo<LAW>::NQ;
    constexpr int S = SOf<RECON>::S;
    if (*done || st->code) return;
    if (st->failures) { st->halt = 1; return; }
    // the faces of one z-slice as one index space (rows of n + 1 or n + 2
    // faces would leave a nearly empty block per row)
    const unsigned lin = blockIdx.x * blockDim.x + threadIdx.x;
    if (lin >= (unsigned) nb0 * (unsigned) nb1) return;
    const int t = (int) (lin % (unsigned) nb0);
    const int i = lo0 + t, j = lo1 + (int) (lin / (unsigned) nb0), k = lo2 + blockIdx.y;
    const long long stride = axis == 0 ? 1 : axis == 1 ? (long long) G.N[0] : (long long) G.N[0] * G.N[1];
    const long long base = ((long long) k * G.N[1] + j) * G.N[0] + i;
    float PL[NQ], PR[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
        float v[2 * S];
#pragma unroll
        for (int c = 0; c < 2 * S; ++c) v[c] = P[q * G.sP + base + (c - S) * stride];
        if constexpr (RECON == RECON_PCM) { PL[q] = v[0]; PR[q] = v[1]; }
        else if constexpr (RECON == RECON_PLM) {
            PL[q] = v[1] + 0.5f * minmod_f(G.plm_theta, v[0], v[1], v[2]);
            PR[q] = v[2] - 0.5f * minmod_f(G.plm_theta, v[1], v[2], v[3]);
        } else {
            PL[q] = weno5_f<true>(&v[2], G.weno_is, G.shenzha_A);
            PR[q] = weno5_f<false>(&v[3], G.weno_is, G.shenzha_A);
        }
    }
    using Normal = std::conditional_t<(AXIS >= 0), AxisNormal<(AXIS >= 0 ? AXIS : 0)>, VecNormal>;
    Normal n;
    if constexpr (AXIS < 0) n.n = G.nrm[axis];
    StateF<NQ> L, R;
    int e = law_prim_f<LAW>(G.gamma, PL, n, L);
    if (e == ST_OK) e = law_prim_f<LAW>(G.gamma, PR, n, R);
    if (e != ST_OK) { atomicCAS(&st->code, 0, e); return; }
    float Fh[NQ];
    if constexpr (RIEMANN == RIEMANN_HLLC) hllc_f<NQ>(L, R, n, Fh);
    else hlle_f<NQ>(L, R, Fh);
    const long long f = ((long long) k * (G.N[1] + 1) + j) * (G.N[0] + 1) + i;
#pragma unroll
    for (int q = 0; q < NQ; ++q) F[q * G.sF + f] = Fh[q];
}

struct FluxViewF {
    const float* F[3];
    const float* E[3];   // edge EMFs of the flux CT (pairs x-y, x-z, y-z), or null
    long long sF;
    int M0, M1;
    __device__ __forceinline__ float at(int a, int q, int i, int j, int k) const
    {
        return F[a][q * sF + ((long long) k * M1 + j) * M0 + i];
    }
    __device__ __forceinline__ float emf(int e, int i, int j, int k) const
    {
        return E[e][((long long) k * M1 + j) * M0 + i];
    }
};

// The edge EMFs of CellCenteredFieldCT::correctGodunovFluxes (Toth 2000,
// eq. 25), each formed once from the four face fluxes around its edge: for
// axes a < b, E_ab at the edge below face index (i, j, k) on both axes is
// (F_a[B_b] + F_a[B_b](-1 along b) - F_b[B_a] - F_b[B_a](-1 along a)) / 4.
// A corrected flux is then the mean of the two EMFs on its face's edges
// (face_flux_f), which is the reference's 1/8-weighted stencil.
__global__ void __launch_bounds__(128) ct_emf_kernel(FluxViewF V, float* E01, float* E02, float* E12, int M0, int M1,
                                                     int M2, int fx, int fy, int fz)
{
    pdl_chain();
    const unsigned L = blockIdx.x * blockDim.x + threadIdx.x;
    if (L >= (unsigned) M0 * (unsigned) M1) return;
    const int i = (int) (L % (unsigned) M0), j = (int) (L / (unsigned) M0), k = blockIdx.y;
    const long long e = ((long long) k * M1 + j) * M0 + i;
    constexpr int B0 = 5, B1 = 6, B2 = 7;
    if (fx && fy && i > 0 && j > 0)
        E01[e] = 0.25f * (V.at(0, B1, i, j, k) + V.at(0, B1, i, j - 1, k) - V.at(1, B0, i, j, k) - V.at(1, B0, i - 1, j, k));
    if (fx && fz && i > 0 && k > 0)
        E02[e] = 0.25f * (V.at(0, B2, i, j, k) + V.at(0, B2, i, j, k - 1) - V.at(2, B0, i, j, k) - V.at(2, B0, i - 1, j, k));
    if (fy && fz && j > 0 && k > 0)
        E12[e] = 0.25f * (V.at(1, B2, i, j, k) + V.at(1, B2, i, j, k - 1) - V.at(2, B1, i, j, k) - V.at(2, B1, i, j - 1, k));
    (void) M2;
}

// flux CT of CellCenteredFieldCT::correctGodunovFluxes on one face (FP32):
// the normal field's flux is zero, a tangential field's the mean of the edge
// EMFs (ct_emf_kernel) on the face's two edges along the other axis
template <int NQ>
__device__ __forceinline__ float face_flux_f(const FluxViewF& V, const GridF& G, int a, int q, int i, int j, int k)
{
    if (NQ == 8 && G.ct && q >= 5) {
        const bool fx = G.n[0] > 1, fy = G.n[1] > 1, fz = G.n[2] > 1;
        const int B0 = 5, B1 = 6, B2 = 7;
        if (a == 0) {
            if (q == B0) return 0.f;
            if (q == B1 && fy) return 0.5f * (V.emf(0, i, j + 1, k) + V.emf(0, i, j, k));
            if (q == B2 && fz) return 0.5f * (V.emf(1, i, j, k + 1) + V.emf(1, i, j, k));
        } else if (a == 1) {
            if (q == B1) return 0.f;
            if (q == B2 && fz) return 0.5f * (V.emf(2, i, j, k + 1) + V.emf(2, i, j, k));
            if (q == B0 && fx) return -0.5f * (V.emf(0, i + 1, j, k) + V.emf(0, i, j, k));
        } else {
            if (q == B2) return 0.f;
            if (q == B0 && fx) return -0.5f * (V.emf(1, i + 1, j, k) + V.emf(1, i, j, k));
            if (q == B1 && fy) return -0.5f * (V.emf(2, i, j + 1, k) + V.emf(2, i, j, k));
        }
    }
    return V.at(a, q, i, j, k);
}

// The 2-D (Z, W) Newton iteration of ConsToPrimRMHD (rm_anton2dzw, after
// ConsToPrimRMHD::solve_anton2dzw, ConsToPrimRMHD.cpp:183-255) in reciprocal
// form for the mixed path: 1/Z and
// 1/W are formed once per iterate (and carried into the next iteration,
// where the convergence test needs them too) and the Jacobian's inverse
// from 1/det, so an iteration divides three times instead of about twenty;
// FP64 division is a long instruction sequence on this GPU.  The update, the
// clamps, the convergence test and the iteration cap are the reference's;
// the iterates differ from the plain path's by rounding only.
// ConsToPrimRMHD::reconstruct_prim (ConsToPrimRMHD.cpp:110-145) from the
// root (Z, W) and their reciprocals, with reciprocals instead of divisions
__device__ __forceinline__ int rm_reconstruct_rcp(const C2pRmhd& s, double Z, double W, double iZ, double iW,
                                                  double* Pout)
{
    double P[8];
    const double iZB = 1.0 / (Z + s.B2);
    const double b0 = s.BS * W * iZ;
    P[0] = s.D * iW;
    P[4] = P[0] * (Z * iW / s.D - 1.0) * s.gamf;
    P[1] = (s.Cons[1] + b0 * s.Cons[5] * iW) * iZB;
    P[2] = (s.Cons[2] + b0 * s.Cons[6] * iW) * iZB;
    P[3] = (s.Cons[3] + b0 * s.Cons[7] * iW) * iZB;
    P[5] = s.Cons[5];
    P[6] = s.Cons[6];
    P[7] = s.Cons[7];
    if (P[4] <= 0.0 && s.pfloor > 0.0) P[4] = P[0] * s.pfloor;
    const int err = rm_check_prim(P);
    if (err) return err;
#pragma unroll
    for (int q = 0; q < 8; ++q) Pout[q] = P[q];
    return ST_OK;
}

__device__ __forceinline__ int rm_anton2dzw_rcp(const C2pRmhd& s, double* P)
{
    const int bad = rm_check_cons(s.Cons);
    if (bad) return bad;
    int it = 0;
    double error = 1.0, W = s.W_start, Z = s.Z_start;
    const double D = s.D, Tau = s.Tau, S2 = s.S2, B2 = s.B2, BS2 = s.BS2, gamf = s.gamf;
    const double iD = 1.0 / D;
    double iW = 1.0 / W, iZ = 1.0 / Z;
    while (error > 1e-12) {
        const double Z2 = Z * Z, Z3 = Z * Z2, W2 = W * W;
        const double iW2 = iW * iW, iW3 = iW2 * iW, iZ2 = iZ * iZ, iZ3 = iZ2 * iZ;
        const double BZ = B2 + Z;
        const double Pre = (D * iW) * (Z * iD * iW - 1.0) * gamf;
        const double df0dZ = 2 * BZ * (BS2 * W2 + (W2 - 1) * Z3) * iW2 * iZ3;
        const double df0dW = 2 * BZ * BZ * iW3;
        const double df1dZ = 1.0 + BS2 * iZ3 - gamf * iW2;
        const double df1dW = B2 * iW3 + (2 * Z - D * W) * iW3 * gamf;
        const double f0 = -S2 + BZ * BZ * (W2 - 1) * iW2 - (2 * Z + B2) * BS2 * iZ2;
        const double f1 = -Tau + Z + B2 - Pre - 0.5 * B2 * iW2 - 0.5 * BS2 * iZ2 - D;
        const double idet = 1.0 / (df0dZ * df1dW - df0dW * df1dZ);
        const double dZ = -(df1dW * f0 - df0dW * f1) * idet;
        const double dW = -(df0dZ * f1 - df1dZ * f0) * idet;
        double Z_new = Z + dZ;
        double W_new = W + dW;
        Z_new = (Z_new > 0.0) ? Z_new : -Z_new;
        Z_new = (Z_new < 1e20) ? Z_new : Z;
        W_new = (W_new > 1.0) ? W_new : 1.0;
        W_new = (W_new < 1e12) ? W_new : 1e12;
        Z = Z_new;
        W = W_new;
        iZ = 1.0 / Z;
        iW = 1.0 / W;
        error = fabs(dZ * iZ) + fabs(dW * iW);
        ++it;
        if (it == 250) return ST_C2P_MAXITER;
    }
    return rm_reconstruct_rcp(s, Z, W, iZ, iW, P);
}

// The same (Z, W) Newton iteration with its residuals f0, f1 formed in FP32
// pairs (about 46 significant bits; FP64 runs at 1/64 of the FP32 rate on
// this GPU) and the 2x2 Jacobian solved in FP32: an approximate Jacobian
// keeps Newton's iteration converging (at rate ~1e-7 once quadratic
// convergence has done its work), and the root is as accurate as the
// residuals.  The reference's start, clamps, convergence test (|dZ/Z| +
// |dW/W| <= 1e-12) and reconstruction (ConsToPrimRMHD.cpp:110-145, 183-255).
// Returns false, leaving P untouched, wherever the pair form cannot be
// trusted to finish as the FP64 iteration would: magnitudes outside
// RM_PAIR_LO..RM_PAIR_HI (the pair's lower word would leave FP32's normal
// range), no convergence within RM_PAIR_MAXIT iterations, a non-finite step,
// or primitives that fail the reference's checks; the caller then runs the
// FP64 solve, which also supplies the reference's error code.
constexpr float RM_PAIR_LO = 1e-8f, RM_PAIR_HI = 1e8f, RM_PAIR_WMAX = 1e4f;
constexpr int RM_PAIR_MAXIT = 16;

__device__ __forceinline__ bool rm_in_range(df x) { return x.hi >= RM_PAIR_LO && x.hi <= RM_PAIR_HI; }

__device__ __forceinline__ bool rm_recover_pair(const GridF& G, const df* U, const float* Pprev, float* Pout)
{
    const df D = U[0], Tau = U[4];
    if (!rm_in_range(D) || !(Tau.hi >= 0.0f && Tau.hi <= RM_PAIR_HI)) return false;
#pragma unroll
    for (int q = 1; q < 8; ++q)
        if (!(fabsf(U[q].hi) <= RM_PAIR_HI)) return false;
    const df S2 = df_add(df_add(df_mul(U[1], U[1]), df_mul(U[2], U[2])), df_mul(U[3], U[3]));
    const df B2 = df_add(df_add(df_mul(U[5], U[5]), df_mul(U[6], U[6])), df_mul(U[7], U[7]));
    const df BS = df_add(df_add(df_mul(U[5], U[1]), df_mul(U[6], U[2])), df_mul(U[7], U[3]));
    const df BS2 = df_mul(BS, BS);
    const df gamf = {G.rm_gamf_hi, G.rm_gamf_lo};
    const df iD = df_rcp(D);
    df Z, W;
    bool warm = false;
    if (Pprev) {
        // warm start from the zone's previous primitives (as the FP64 solve)
        const float rho = Pprev[0], pre = Pprev[4];
        const df V2 = df_add(df_add(two_prod(Pprev[1], Pprev[1]), two_prod(Pprev[2], Pprev[2])),
                             two_prod(Pprev[3], Pprev[3]));
        if (rho > 0.0f && pre > 0.0f && V2.hi < 1.0f) {
            const df W2 = df_rcp(df_add_f(df_neg(V2), 1.0f));
            const float h = 1.0f + pre * rcp_approx(rho) * G.rm_hcoef;
            Z = df_mul_f(W2, rho * h);
            W = df_sqrt(W2);
            warm = true;
        }
    }
    if (!warm) {  // the cold start of ConsToPrimRMHD::estimate_from_cons
        Z = df_sqrt(df_add(S2, df_mul(D, D)));
        W = df_mul(Z, iD);
    }
    if (!rm_in_range(Z) || !(W.hi >= 0.5f && W.hi <= RM_PAIR_WMAX)) return false;
    const df hB2 = df_pow2(B2, 0.5f), hBS2 = df_pow2(BS2, 0.5f);
    df iZ = df_rcp(Z), iW = df_rcp(W);
    float error = 1.0f;
    int it = 0;
    while (error > 1e-12f) {
        if (++it > RM_PAIR_MAXIT) return false;
        const df W2 = df_mul(W, W), W2m1 = df_add_f(W2, -1.0f);
        const df iW2 = df_mul(iW, iW), iZ2 = df_mul(iZ, iZ);
        const df BZ = df_add(B2, Z);
        // f0 = -S2 + (Z + B2)^2 (W^2 - 1) / W^2 - (2 Z + B2) BS2 / Z^2
        const df f0 = df_sub(df_mul(df_mul(df_mul(BZ, BZ), W2m1), iW2),
                             df_add(S2, df_mul(df_mul(df_add(df_pow2(Z, 2.0f), B2), BS2), iZ2)));
        // f1 = -Tau + Z + B2 - Pre - B2 / (2 W^2) - BS2 / (2 Z^2) - D,
        // Pre = (D / W) (Z / (D W) - 1) gamf
        const df Pre = df_mul(df_mul(D, iW), df_mul(df_add_f(df_mul(df_mul(Z, iD), iW), -1.0f), gamf));
        df f1 = df_sub(df_sub(Z, D), Tau);
        f1 = df_sub(df_add(f1, B2), Pre);
        f1 = df_sub(df_sub(f1, df_mul(hB2, iW2)), df_mul(hBS2, iZ2));
        // the Jacobian, in FP32
        const float z = Z.hi, w = W.hi, iz = iZ.hi, iw = iW.hi, g = gamf.hi;
        const float bz = BZ.hi, iw2 = iw * iw, iw3 = iw2 * iw, iz3 = iz * iz * iz, z3 = z * z * z;
        const float j00 = 2.0f * bz * (BS2.hi * W2.hi + W2m1.hi * z3) * iw2 * iz3;
        const float j01 = 2.0f * bz * bz * iw3;
        const float j10 = 1.0f + BS2.hi * iz3 - g * iw2;
        const float j11 = B2.hi * iw3 + (2.0f * z - D.hi * w) * iw3 * g;
        const float idet = rcp_approx(j00 * j11 - j01 * j10);
        const float dZ = -(j11 * f0.hi - j01 * f1.hi) * idet;
        const float dW = -(j00 * f1.hi - j10 * f0.hi) * idet;
        if (!isfinite(dZ) || !isfinite(dW)) return false;
        df Zn = df_add_f(Z, dZ), Wn = df_add_f(W, dW);
        if (Zn.hi < 0.0f) Zn = df_neg(Zn);
        if (Wn.hi < 1.0f || (Wn.hi == 1.0f && Wn.lo < 0.0f)) Wn = {1.0f, 0.0f};
        if (!rm_in_range(Zn) || Wn.hi > RM_PAIR_WMAX) return false;
        Z = Zn;
        W = Wn;
        iZ = df_rcp(Z);
        iW = df_rcp(W);
        error = fabsf(dZ * iZ.hi) + fabsf(dW * iW.hi);
    }
    // reconstruction, checked as ConsToPrimRMHD::check_prim does
    const df iZB = df_rcp(df_add(Z, B2));
    const df b0 = df_mul(df_mul(BS, W), iZ);
    const df rho = df_mul(D, iW);
    df pre = df_mul(df_mul(rho, df_add_f(df_mul(df_mul(Z, iW), iD), -1.0f)), gamf);
    if (pre.hi <= 0.0f && G.pressure_floor > 0.0f) pre = df_mul_f(rho, G.pressure_floor);
    df v[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) v[a] = df_mul(df_add(U[1 + a], df_mul(df_mul(b0, U[5 + a]), iW)), iZB);
    const df v2 = df_add(df_add(df_mul(v[0], v[0]), df_mul(v[1], v[1])), df_mul(v[2], v[2]));
    if (!(v2.hi < 1.0f) || pre.hi < 0.0f || rho.hi < 0.0f) return false;
    float P[8];
    P[0] = __fadd_rn(rho.hi, rho.lo);
    P[1] = __fadd_rn(v[0].hi, v[0].lo);
    P[2] = __fadd_rn(v[1].hi, v[1].lo);
    P[3] = __fadd_rn(v[2].hi, v[2].lo);
    P[4] = __fadd_rn(pre.hi, pre.lo);
#pragma unroll
    for (int q = 5; q < 8; ++q) P[q] = __fadd_rn(U[q].hi, U[q].lo);
#pragma unroll
    for (int q = 0; q < 8; ++q)
        if (!isfinite(P[q])) return false;
#pragma unroll
    for (int q = 0; q < 8; ++q) Pout[q] = P[q];
    return true;
}

// the relativistic recovery's FP64 ConsToPrimRMHD solve (ConsToPrimRMHD.cpp:
// 183-323) from FP64 conserved densities
__device__ __forceinline__ int recover_rmhd_fp64(const GridF& G, const double* U, float* P, int* code,
                                                 const float* Pprev)
{
    constexpr int NQ = 8;
    {
        double Pd[NQ];
        PhysParams pp;
        pp.gamma = G.gamma_d;
        pp.pressure_floor = G.pfloor_d;
        pp.plm_theta = 0.0;
        pp.shenzha_A = 0.0;
        pp.weno_is = 0;
        // the Newton solve, without the eigenvalue evaluation of the closing
        // fromPrimitive call (its FP32 counterpart runs in the flux kernels)
        C2pRmhd s;
        s.gamf = (pp.gamma - 1.0) / pp.gamma;
        s.pfloor = pp.pressure_floor;
        s.D = U[0];
        s.Tau = U[4];
        s.S2 = U[1] * U[1] + U[2] * U[2] + U[3] * U[3];
        s.B2 = U[5] * U[5] + U[6] * U[6] + U[7] * U[7];
        s.BS = U[5] * U[1] + U[6] * U[2] + U[7] * U[3];
        s.BS2 = s.BS * s.BS;
#pragma unroll
        for (int q = 0; q < 8; ++q) s.Cons[q] = U[q];
        bool warm = false;
        if (Pprev) {
            // warm start from the zone's primitives of the previous stage
            // (ConsToPrimRMHD::set_starting_prim, ConsToPrimRMHD.cpp:99-108):
            // Z = rho h W^2 and W of the old state are close to the new root
            const double rho = f2d_exact(Pprev[0]), pre = f2d_exact(Pprev[4]);
            const double v1 = f2d_exact(Pprev[1]), v2 = f2d_exact(Pprev[2]), v3 = f2d_exact(Pprev[3]);
            const double V2 = v1 * v1 + v2 * v2 + v3 * v3;
            if (rho > 0.0 && pre > 0.0 && V2 < 1.0) {
                const double W2 = 1.0 / (1.0 - V2);
                const double h = 1.0 + pre / rho * (G.inv_gm1_d + 1.0);
                s.Z_start = rho * h * W2;
                s.W_start = sqrt(W2);
                warm = true;
            }
        }
        if (!warm) {
            // the cold start of ConsToPrimRMHD::estimate_from_cons (ConsToPrimRMHD.cpp:88-92)
            s.Z_start = sqrt(s.S2 + s.D * s.D);
            s.W_start = s.Z_start / s.D;
        }
        int err = rm_anton2dzw_rcp(s, Pd);
        if (err != ST_OK) err = rm_noble1dw(s, Pd);
        if (err != ST_OK) { *code = err; return ST_INVERSION_FAILURE; }
#pragma unroll
        for (int q = 0; q < NQ; ++q) P[q] = d2f_rn_ftz(Pd[q]);
        return ST_OK;
    }
}

// FP32 recovery of hydro and MHD from FP32 conserved densities
template <int LAW>
__device__ __forceinline__ int recover_f32(const GridF& G, const float* U, float* P, int* code)
{
    if constexpr (LAW == LAW_HYDRO) {
        hydro_cons_f(G.gamma, U, P);
        return ST_OK;
    } else {
        const int e = mhd_cons_f(G.gamma, G.pressure_floor, U, P);
        *code = e;
        return e;
    }
}

// primitive recovery of the mixed path: FP32 for hydro and MHD; for RMHD the
// pair-residual Newton iteration above, else the FP64 ConsToPrimRMHD solve
template <int LAW>
__device__ __forceinline__ int recover_mixed(const GridF& G, const df* Un, float* P, int* code, const float* Pprev = nullptr)
{
    constexpr int NQ = LawInfo<LAW>::NQ;
    if constexpr (LAW != LAW_RMHD) {
        float U[NQ];
#pragma unroll
        for (int q = 0; q < NQ; ++q) U[q] = Un[q].hi + Un[q].lo;
        return recover_f32<LAW>(G, U, P, code);
    } else {
        if (rm_recover_pair(G, Un, Pprev, P)) return ST_OK;
        double U[NQ];
#pragma unroll
        for (int q = 0; q < NQ; ++q) U[q] = df_to_double(Un[q]);
        return recover_rmhd_fp64(G, U, P, code, Pprev);
    }
}

// the recovery with the FP64 accumulator: FP32 for hydro and MHD (from the
// accumulator rounded to FP32), the FP64 Newton solve for RMHD
template <int LAW>
__device__ __forceinline__ int recover_acc64(const GridF& G, const double* Un, float* P, int* code,
                                             const float* Pprev = nullptr)
{
    constexpr int NQ = LawInfo<LAW>::NQ;
    if constexpr (LAW != LAW_RMHD) {
        float U[NQ];
#pragma unroll
        for (int q = 0; q < NQ; ++q) U[q] = d2f_rn_ftz(Un[q]);
        return recover_f32<LAW>(G, U, P, code);
    } else {
        return recover_rmhd_fp64(G, Un, P, code, Pprev);
    }
}

// Courant step of one zone from its FP32 primitives: lmin / the largest
// |eigenvalue| over the three face normals (FieldOperator::getCourantTimestep,
// FieldOperator.cpp:125-169); an eigenvalue error goes to the status
template <int LAW>
__device__ __forceinline__ float zone_dt_f(const GridF& G, const float* P, DevStatus* st)
{
    constexpr int NQ = LawInfo<LAW>::NQ;
    float lmax = 0.f;
    for (int a = 0; a < 3; ++a) {
        StateF<NQ> S;
        const int e = law_prim_f<LAW>(G.gamma, P, VecNormal{G.nrm[a]}, S);
        if (e != ST_OK) { atomicCAS(&st->code, 0, e); return 3.0e38f; }
        lmax = fmaxf(lmax, fmaxf(fabsf(S.amax), fabsf(S.amin)));
    }
    return G.lmin / lmax;
}

// One RK stage's update of the general form: divergence of the (flux-CT
// corrected) face fluxes, the RK combine on FP32 pairs, the primitive
// recovery, the primitives with their guard images, and on the last stage
// (cfl not null) the zone's Courant step.  Every load of a zone comes before
// its first store, so the loads of all fields are in flight together (the
// stage input and output may be one array, RK1).  Eight blocks per SM: the
// kernel is bound by memory latency, and 32 resident warps with a few spilled
// registers beat 20 warps without (MHD 256^3: 2.34e9 -> 2.64e9 zone-updates/s).
template <int LAW, bool ACC64>
__global__ void __launch_bounds__(128, 8) update_f_kernel(float* __restrict__ Pf, const float* U0h, const float* U0l,
                                                       const float* Uph, const float* Upl, float* Unh, float* Unl,
                                                       FluxViewF V, GridF G,
                                                       const double* __restrict__ dtp, float b, float omb,
                                                       const int* __restrict__ done, DevStatus* st,
                                                       unsigned long long* cfl)
{
    constexpr int NQ = LawInfo<LAW>::NQ;
    pdl_chain();
    if (*done || st->code || st->halt) return;
    const int ii = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = ii < G.n[0];
    const int jj = blockIdx.y, kk = blockIdx.z;
    const int i = ii + G.g[0], j = jj + G.g[1], k = kk + G.g[2];
    const long long uc = ((long long) kk * G.n[1] + jj) * G.n[0] + ii;
    const long long pc = ((long long) k * G.N[1] + j) * G.N[0] + i;
    float Pn[NQ];
    float zdt = 3.0e38f;
    if (active) {
        const float dt = (float) *dtp;
        const bool fx = G.n[0] > 1, fy = G.n[1] > 1, fz = G.n[2] > 1;
        // FP32 pairs, or FP64 (ACC64: the arrays Uh hold doubles)
        using Acc = std::conditional_t<ACC64, double, df>;
        Acc U0[NQ], Up[NQ];
        float L[NQ];
        // the zone's previous primitives: the RMHD recovery's starting point,
        // and what a failed recovery keeps (read only then for the other laws)
        float Pold[NQ];
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
            if constexpr (ACC64) {
                U0[q] = reinterpret_cast<const double*>(U0h)[q * G.sU + uc];
                Up[q] = reinterpret_cast<const double*>(Uph)[q * G.sU + uc];
            } else {
                U0[q] = {U0h[q * G.sU + uc], U0l[q * G.sU + uc]};
                Up[q] = {Uph[q * G.sU + uc], Upl[q * G.sU + uc]};
            }
            if constexpr (LAW == LAW_RMHD) Pold[q] = Pf[q * G.sP + pc];
        }
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
            float l = 0.f;
            if (fx) l -= (face_flux_f<NQ>(V, G, 0, q, i + 1, j, k) - face_flux_f<NQ>(V, G, 0, q, i, j, k)) * G.idx[0];
            if (fy) l -= (face_flux_f<NQ>(V, G, 1, q, i, j + 1, k) - face_flux_f<NQ>(V, G, 1, q, i, j, k)) * G.idx[1];
            if (fz) l -= (face_flux_f<NQ>(V, G, 2, q, i, j, k + 1) - face_flux_f<NQ>(V, G, 2, q, i, j, k)) * G.idx[2];
            L[q] = l;
        }
        Acc Un[NQ];
        int code = ST_OK;
        int e;
        if constexpr (ACC64) {
#pragma unroll
            for (int q = 0; q < NQ; ++q) Un[q] = rk_combine_d(U0[q], Up[q], dt * L[q], b);
#pragma unroll
            for (int q = 0; q < NQ; ++q) reinterpret_cast<double*>(Unh)[q * G.sU + uc] = Un[q];
            e = recover_acc64<LAW>(G, Un, Pn, &code, LAW == LAW_RMHD ? Pold : nullptr);
        } else {
#pragma unroll
            for (int q = 0; q < NQ; ++q) Un[q] = rk_combine(U0[q], Up[q], dt * L[q], b, omb);
#pragma unroll
            for (int q = 0; q < NQ; ++q) {
                Unh[q * G.sU + uc] = Un[q].hi;
                Unl[q * G.sU + uc] = Un[q].lo;
            }
            e = recover_mixed<LAW>(G, Un, Pn, &code, LAW == LAW_RMHD ? Pold : nullptr);
        }
        if (e == ST_INVERSION_FAILURE) {
            atomicAdd(&st->failures, 1);
            const unsigned long long z = (unsigned long long) uc;
            const unsigned long long prev = atomicMin(&st->first_zone, z);
            if (z < prev) atomicExch(&st->first_code, code);
#pragma unroll
            for (int q = 0; q < NQ; ++q) Pn[q] = LAW == LAW_RMHD ? Pold[q] : Pf[q * G.sP + pc];
        }
        if (cfl) zdt = zone_dt_f<LAW>(G, Pn, st);
    }
    // every lane of a warp reaches the reduction (cfl is the same for all)
    if (cfl) block_min_to(cfl, zdt);
    if (!active) return;
    // the zone's cell, then (zones within a guard width of an edge) its guard
    // images on every combination of axes
#pragma unroll
    for (int q = 0; q < NQ; ++q) Pf[q * G.sP + pc] = Pn[q];
    const bool edge = (G.g[0] && (ii < G.g[0] || ii >= G.n[0] - G.g[0])) ||
                      (G.g[1] && (jj < G.g[1] || jj >= G.n[1] - G.g[1])) ||
                      (G.g[2] && (kk < G.g[2] || kk >= G.n[2] - G.g[2]));
    if (!edge) return;
    for (int c = 0; c <= G.g[2]; ++c) {
        int oz, sz;
        if (!guard_image(c, kk, G.n[2], G.g[2], G.bc, oz, sz)) continue;
        for (int bb = 0; bb <= G.g[1]; ++bb) {
            int oy, sy;
            if (!guard_image(bb, jj, G.n[1], G.g[1], G.bc, oy, sy)) continue;
            for (int a = 0; a <= G.g[0]; ++a) {
                int ox, sx;
                if ((a | bb | c) == 0 || !guard_image(a, ii, G.n[0], G.g[0], G.bc, ox, sx)) continue;
                const long long o = ((long long) oz * G.N[1] + oy) * G.N[0] + ox;
#pragma unroll
                for (int q = 0; q < NQ; ++q) {
                    float v = Pn[q];
                    if ((q == 1 && sx) || (q == 2 && sy) || (q == 3 && sz)) v = -v;
                    Pf[q * G.sP + o] = v;
                }
            }
        }
    }
}

template <int LAW>
__global__ void __launch_bounds__(256) courant_f_kernel(const float* __restrict__ Pf, GridF G,
                                                        unsigned long long* __restrict__ dst, DevStatus* st)
{
    constexpr int NQ = LawInfo<LAW>::NQ;
    const int ii = blockIdx.x * blockDim.x + threadIdx.x;
    float zdt = 3.0e38f;
    if (ii < G.n[0]) {
        const long long pc = ((long long) (blockIdx.z + G.g[2]) * G.N[1] + (blockIdx.y + G.g[1])) * G.N[0] + (ii + G.g[0]);
        float P[NQ];
#pragma unroll
        for (int q = 0; q < NQ; ++q) P[q] = Pf[q * G.sP + pc];
        float lmax = 0.f;
        for (int a = 0; a < 3; ++a) {
            StateF<NQ> S;
            const int e = law_prim_f<LAW>(G.gamma, P, VecNormal{G.nrm[a]}, S);
            if (e != ST_OK) { atomicCAS(&st->code, 0, e); break; }
            lmax = fmaxf(lmax, fmaxf(fabsf(S.amax), fabsf(S.amin)));
        }
        zdt = G.lmin / lmax;
    }
    block_min_to(dst, zdt);
}

// AoS FP64 MeshData::P (cells [c0, c1)) -> FP32-pair conserved state and,
// on the general form, FP32 primitives with guards.  Hydro converts with one
// reciprocal instead of FP64 divisions (FP64 is slow on this GPU) and, when
// cfl is given, reduces the Courant step of the loaded zones on the way.
//
// A block's cells are one contiguous slab of the AoS array: it is read with
// consecutive threads on consecutive doubles (the array may be the caller's
// page-locked host memory, read over the chip-to-chip link, where scattered
// per-cell accesses are slow) and transposed to cells in shared memory.
constexpr int CONV_BLOCK = 256;

template <int LAW, bool ACC64>
__global__ void __launch_bounds__(CONV_BLOCK) load_kernel(const double* __restrict__ aos, long long c0, long long c1,
                                                          float* Uh, float* Ul, float* Pf, GridF G, PhysParams pp,
                                                          DevStatus* st, unsigned long long* cfl)
{
    constexpr int NQ = LawInfo<LAW>::NQ;
    __shared__ double slab[CONV_BLOCK * NQ];
    const long long b0 = c0 + blockIdx.x * (long long) CONV_BLOCK;
    const int nc = (int) min((long long) CONV_BLOCK, c1 - b0);
    for (int e = threadIdx.x; e < nc * NQ; e += CONV_BLOCK) slab[e] = aos[b0 * NQ + e];
    __syncthreads();
    const long long c = b0 + threadIdx.x;
    float zdt = 3.0e38f;
    if (threadIdx.x < nc) {
        const int k = (int) (c % G.N[2]);
        const int j = (int) ((c / G.N[2]) % G.N[1]);
        const int i = (int) (c / ((long long) G.N[2] * G.N[1]));
        double P[NQ];
#pragma unroll
        for (int q = 0; q < NQ; ++q) P[q] = slab[threadIdx.x * NQ + q];
        const long long s = ((long long) k * G.N[1] + j) * G.N[0] + i;
        if (Pf)
#pragma unroll
            for (int q = 0; q < NQ; ++q) Pf[q * G.sP + s] = (float) P[q];
        const int ii = i - G.g[0], jj = j - G.g[1], kk = k - G.g[2];
        if (ii >= 0 && jj >= 0 && kk >= 0 && ii < G.n[0] && jj < G.n[1] && kk < G.n[2]) {
            double U[NQ];
            if constexpr (LAW == LAW_HYDRO) {
                hydro_p2u_d(P, G.inv_gm1_d, U);
            } else {
                const int e = law_p2u<LAW>(pp, P, U);
                if (e != ST_OK) atomicCAS(&st->code, 0, e);
            }
            const long long u = ((long long) kk * G.n[1] + jj) * G.n[0] + ii;
            float hi[NQ];
#pragma unroll
            for (int q = 0; q < NQ; ++q) {
                if constexpr (ACC64) {
                    reinterpret_cast<double*>(Uh)[q * G.sU + u] = U[q];
                    hi[q] = d2f_rn_ftz(U[q]);
                    if (Ul) Ul[q * G.sU + u] = hi[q];   // the fused form's FP32 copy
                } else {
                    const df d = df_from_double(U[q]);
                    Uh[q * G.sU + u] = d.hi;
                    Ul[q * G.sU + u] = d.lo;
                    hi[q] = d.hi;
                }
            }
            // the Courant step from the stored high words, as the last RK
            // stage computes it
            if constexpr (LAW == LAW_HYDRO)
                if (cfl) zdt = hydro_zone_dt(G.gamma, G.lmin, hi);
        }
    }
    if (cfl) block_min_to(cfl, zdt);
}

// FP64 primitives of cell c (AoS order) from the FP32-pair state; a guard
// zone is the boundary image of an interior zone
template <int LAW, bool L2ONLY = false, bool ACC64 = false>
__device__ __forceinline__ void store_cell(const float* Uh, const float* Ul, long long c, const GridF& G,
                                           const PhysParams& pp, double* out)
{
    constexpr int NQ = LawInfo<LAW>::NQ;
    const int k = (int) (c % G.N[2]);
    const int j = (int) ((c / G.N[2]) % G.N[1]);
    const int i = (int) (c / ((long long) G.N[2] * G.N[1]));
    int f[3] = {0, 0, 0};
    const int ii = G.n[0] > 1 ? bc_image(i - G.g[0], G.n[0], G.bc, f[0]) : 0;
    const int jj = G.n[1] > 1 ? bc_image(j - G.g[1], G.n[1], G.bc, f[1]) : 0;
    const int kk = G.n[2] > 1 ? bc_image(k - G.g[2], G.n[2], G.bc, f[2]) : 0;
    const long long u = ((long long) kk * G.n[1] + jj) * G.n[0] + ii;
    double U[NQ], P[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
        if constexpr (ACC64) U[q] = reinterpret_cast<const double*>(Uh)[q * G.sU + u];
        else U[q] = f2d_exact(ld_state<L2ONLY>(Uh + q * G.sU + u)) + f2d_exact(ld_state<L2ONLY>(Ul + q * G.sU + u));
    }
    if constexpr (LAW == LAW_HYDRO) {
        hydro_u2p_d(U, G.gm1_d, P);
    } else {
        int code = 0;
        law_cons<LAW>(pp, U, P, &code);
    }
    if (f[0]) P[1] = -P[1];
    if (f[1]) P[2] = -P[2];
    if (f[2]) P[3] = -P[3];
#pragma unroll
    for (int q = 0; q < NQ; ++q) out[q] = P[q];
}

// FP32-pair state -> AoS FP64 primitives with guards, cells [c0, c1), each
// block's slab written as one contiguous run
template <int LAW, bool ACC64>
__global__ void __launch_bounds__(CONV_BLOCK) store_kernel(const float* Uh, const float* Ul, double* __restrict__ aos,
                                                           long long c0, long long c1, GridF G, PhysParams pp)
{
    constexpr int NQ = LawInfo<LAW>::NQ;
    __shared__ double slab[CONV_BLOCK * NQ];
    const long long b0 = c0 + blockIdx.x * (long long) CONV_BLOCK;
    const int nc = (int) min((long long) CONV_BLOCK, c1 - b0);
    if (threadIdx.x < nc) store_cell<LAW, false, ACC64>(Uh, Ul, b0 + threadIdx.x, G, pp, &slab[threadIdx.x * NQ]);
    __syncthreads();
    for (int e = threadIdx.x; e < nc * NQ; e += CONV_BLOCK) aos[b0 * NQ + e] = slab[e];
}

// The step-start kernels let the stage launched after them start at once
// (programmatic dependent launch): its staging and faces need nothing they
// write, and it waits for them before its update.
__device__ __forceinline__ void release_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

__global__ void k_cfl_reset(unsigned long long* bits)
{
    pdl_chain();
    *bits = (unsigned long long) __double_as_longlong(DBL_MAX);
}
__global__ void k_cfl_publish(const unsigned long long* bits, DevStatus* st) { st->dt_bits = *bits; }
// RK1 on the fused path alternates the state buffer; a step that found the
// loop done (or an error) did no work and keeps it
__global__ void k_rot_flip(int* rot, const DevStatus* st)
{
    if (!st->done && !st->code) *rot ^= 1;
}
// the general form's last stage reduced the new state's Courant step into
// next; it becomes the handle's only if the step ran (a step not taken, at
// t_final or after an error, leaves the previous state's step)
__global__ void k_cfl_commit(unsigned long long* bits, const unsigned long long* next, const DevStatus* st)
{
    pdl_chain();
    if (!st->done && !st->code && !st->halt) *bits = *next;
}

// Start of one driver-loop step of the fused path, in one thread: the Courant
// step that the previous step's last stage (or the load) reduced becomes the
// handle's, dt = min(cfl x courant, t_final - t) (src/Problems.cpp:181-186),
// the reduction slot is reset for this step's last stage, and the clock
// advances (the fused hydro stages record no inversion failures, so the step
// cannot fail after this point).
__global__ void k_fused_run_begin(unsigned long long* bits, DevStatus* st, double cfl, double t_final)
{
    release_dependents();
    if (st->done) return;
    st->dt_bits = *bits;
    double dt = cfl * __longlong_as_double((long long) st->dt_bits);
    if (t_final >= 0.0) {
        if (!(st->t < t_final)) { st->done = 1; return; }
        const double dt2 = t_final - st->t;
        dt = dt < dt2 ? dt : dt2;
    }
    st->dt = dt;
    *bits = (unsigned long long) __double_as_longlong(DBL_MAX);
    if (st->code) return;
    st->t += dt;
    st->steps += 1;
}

// Start of one advance with a given dt on the fused path.
__global__ void k_fused_advance_begin(unsigned long long* bits, DevStatus* st, double dt)
{
    release_dependents();
    st->done = 0;   // an advance with a given dt is always taken
    st->dt = dt;
    *bits = (unsigned long long) __double_as_longlong(DBL_MAX);
}

// ---------------------------------------------------------------------------
struct MixedState {
    MaraGpuConfig cfg;
    GridDesc G;
    GridF GF;
    PhysParams pp;
    bool fused = false;
    bool acc64 = false;      // MARA_PRECISION_MIXED_FP64: Uh hold FP64 accumulators
    float* Uh[3] = {nullptr, nullptr, nullptr};
    float* Ul[3] = {nullptr, nullptr, nullptr};
    float* Pf = nullptr;
    float* F[3] = {nullptr, nullptr, nullptr};
    float* E[3] = {nullptr, nullptr, nullptr};  // flux-CT edge EMFs (magnetic laws)
    HGrid* dgrid = nullptr;
    TileRef* dtiles = nullptr;
    int ntiles = 0;
    int* dntiles = nullptr;
    int* drot = nullptr;     // state buffer index (device)
    int rot = 0;             // host mirror for the general form's parity
    unsigned long long* dcfl = nullptr;
    unsigned long long* dcfl_next = nullptr;  // general form: the last stage's Courant reduction
    int tx = 32, ty = 16;
    int ctas = 0;
    int timing = 0;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev;
    double ms = 0;
    int64_t nlaunch = 0;
    struct HostStep* hs = nullptr;   // the pipelined host step (created on first use)
    bool hs_unavailable = false;     // it could not be set up or launched here
};

static void host_step_destroy(HostStep* hs);

static int dev_alloc(void** p, size_t bytes, cudaStream_t s, int64_t* total)
{
    if (cudaMalloc(p, bytes) != cudaSuccess) return MARA_ERR_CUDA;
    cudaMemsetAsync(*p, 0, bytes, s);
    *total += (int64_t) bytes;
    return MARA_OK;
}

int mixed_create(const MaraGpuConfig* c, const GridDesc& G, MixedState** out, cudaStream_t s, int64_t* bytes)
{
    MixedState* m = new MixedState();
    m->cfg = *c;
    m->G = G;
    GridF& F = m->GF;
    for (int a = 0; a < 3; ++a) {
        F.n[a] = G.n[a]; F.g[a] = G.g[a]; F.N[a] = G.N[a];
        for (int b = 0; b < 3; ++b) F.nrm[a][b] = (float) G.nrm[a][b];
        const double dx = (c->upper[a] - c->lower[a]) / G.n[a];
        F.idx[a] = (float) (1.0 / dx);
    }
    F.sP = G.sP; F.sU = G.sU; F.sF = G.sF;
    F.lmin = (float) G.lmin;
    F.bc = G.bc; F.ct = G.ct;
    F.gamma = (float) c->gamma; F.plm_theta = (float) c->plm_theta; F.shenzha_A = (float) c->shenzha_A;
    F.pressure_floor = (float) c->pressure_floor; F.weno_is = c->weno_is;
    F.gamma_d = c->gamma; F.pfloor_d = c->pressure_floor;
    F.gm1_d = c->gamma - 1.0; F.inv_gm1_d = 1.0 / (c->gamma - 1.0);
    {
        const double gamf = (c->gamma - 1.0) / c->gamma;
        F.rm_gamf_hi = (float) gamf;
        F.rm_gamf_lo = (float) (gamf - (double) F.rm_gamf_hi);
        F.rm_hcoef = (float) (c->gamma / (c->gamma - 1.0));
    }
    m->pp.gamma = c->gamma; m->pp.plm_theta = c->plm_theta; m->pp.shenzha_A = c->shenzha_A;
    m->pp.pressure_floor = c->pressure_floor; m->pp.weno_is = c->weno_is;

    m->fused = c->law == MARA_LAW_HYDRO && G.n[2] == 1 && c->recon != MARA_RECON_WENO5 && G.n[0] > 1;
    m->acc64 = c->precision == MARA_PRECISION_MIXED_FP64;
    const int nq = G.nq;
    int rc = MARA_OK;
    for (int b = 0; b < 3 && !rc; ++b) {
        if (m->acc64) {
            rc = dev_alloc((void**) &m->Uh[b], sizeof(double) * G.sU * nq, s, bytes);
            // the fused form also keeps the accumulator rounded to FP32, which
            // the next stage's halo staging reads (no conversions there)
            if (!rc && m->fused) rc = dev_alloc((void**) &m->Ul[b], sizeof(float) * G.sU * nq, s, bytes);
        } else {
            rc = dev_alloc((void**) &m->Uh[b], sizeof(float) * G.sU * nq, s, bytes);
            if (!rc) rc = dev_alloc((void**) &m->Ul[b], sizeof(float) * G.sU * nq, s, bytes);
        }
    }
    if (!rc) rc = dev_alloc((void**) &m->drot, sizeof(int), s, bytes);
    if (!rc) rc = dev_alloc((void**) &m->dcfl, sizeof(unsigned long long), s, bytes);
    if (!rc && !m->fused) {
        rc = dev_alloc((void**) &m->Pf, sizeof(float) * G.sP * nq, s, bytes);
        if (!rc) rc = dev_alloc((void**) &m->dcfl_next, sizeof(unsigned long long), s, bytes);
        for (int a = 0; a < 3 && !rc; ++a)
            if (G.n[a] > 1) rc = dev_alloc((void**) &m->F[a], sizeof(float) * G.sF * nq, s, bytes);
        if (G.ct && nq == 8)
            for (int e = 0; e < 3 && !rc; ++e) rc = dev_alloc((void**) &m->E[e], sizeof(float) * G.sF, s, bytes);
    }
    if (!rc && m->fused) {
        HGrid h;
        std::memset(&h, 0, sizeof(h));
        for (int b = 0; b < 3; ++b) { h.Uh[b] = m->Uh[b]; h.Ul[b] = m->Ul[b]; }
        h.sU = G.sU;
        h.n0 = G.n[0];
        h.n1 = G.n[1];
        h.bc = G.bc;
        h.gamma = (float) c->gamma;
        h.plm_theta = (float) c->plm_theta;
        h.idx = F.idx[0];
        h.idy = F.idx[1];
        h.lmin = F.lmin;
        m->tx = G.n[1] > 1 ? 32 : 256;
        m->ty = G.n[1] > 1 ? 16 : 1;
        std::vector<TileRef> tiles;
        for (int y = 0; y < G.n[1]; y += m->ty)
            for (int x = 0; x < G.n[0]; x += m->tx) tiles.push_back({0, x, y, 0});
        m->ntiles = (int) tiles.size();
        rc = dev_alloc((void**) &m->dgrid, sizeof(HGrid), s, bytes);
        if (!rc) rc = dev_alloc((void**) &m->dntiles, sizeof(int), s, bytes);
        if (!rc) cudaMemcpyAsync(m->dntiles, &m->ntiles, sizeof(int), cudaMemcpyHostToDevice, s);
        if (!rc) rc = dev_alloc((void**) &m->dtiles, sizeof(TileRef) * tiles.size(), s, bytes);
        if (!rc) {
            cudaMemcpyAsync(m->dgrid, &h, sizeof(HGrid), cudaMemcpyHostToDevice, s);
            cudaMemcpyAsync(m->dtiles, tiles.data(), sizeof(TileRef) * tiles.size(), cudaMemcpyHostToDevice, s);
            cudaStreamSynchronize(s);
        }
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        m->ctas = m->ntiles;
    }
    if (rc) { mixed_destroy(m); return rc; }
    *out = m;
    return MARA_OK;
}

void mixed_destroy(MixedState* m)
{
    if (!m) return;
    for (auto& e : m->ev) { cudaEventDestroy(e.first); cudaEventDestroy(e.second); }
    for (int b = 0; b < 3; ++b) { cudaFree(m->Uh[b]); cudaFree(m->Ul[b]); }
    cudaFree(m->drot); cudaFree(m->dcfl); cudaFree(m->dcfl_next);
    cudaFree(m->Pf);
    for (int a = 0; a < 3; ++a) cudaFree(m->F[a]);
    for (int e = 0; e < 3; ++e) cudaFree(m->E[e]);
    cudaFree(m->dgrid);
    cudaFree(m->dtiles);
    cudaFree(m->dntiles);
    host_step_destroy(m->hs);
    delete m;
}

template <typename Fn>
static void timed(MixedState* m, cudaStream_t s, Fn fn)
{
    if (!m->timing) { fn(); return; }
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a, s);
    fn();
    cudaEventRecord(b, s);
    m->ev.push_back({a, b});
}

static int host_rot(const MixedState* m) { return m->rot; }

static void courant_general(MixedState* m, DevStatus* st, cudaStream_t s)
{
    dim3 grid((m->G.n[0] + 255) / 256, m->G.n[1], m->G.n[2]);
    switch (m->cfg.law) {
        case MARA_LAW_HYDRO: courant_f_kernel<LAW_HYDRO><<<grid, 256, 0, s>>>(m->Pf, m->GF, m->dcfl, st); break;
        case MARA_LAW_MHD: courant_f_kernel<LAW_MHD><<<grid, 256, 0, s>>>(m->Pf, m->GF, m->dcfl, st); break;
        default: courant_f_kernel<LAW_RMHD><<<grid, 256, 0, s>>>(m->Pf, m->GF, m->dcfl, st); break;
    }
}

void mixed_load_begin(MixedState* m, cudaStream_t s)
{
    cudaMemcpyAsync(m->drot, &m->rot, sizeof(int), cudaMemcpyHostToDevice, s);
    k_cfl_reset<<<1, 1, 0, s>>>(m->dcfl);
}

template <bool ACC64>
static void load_range(MixedState* m, const double* aos, long long c0, long long c1, DevStatus* st, cudaStream_t s)
{
    const int r = host_rot(m);
    const unsigned nb = (unsigned) ((c1 - c0 + 255) / 256);
    switch (m->cfg.law) {
        case MARA_LAW_HYDRO:
            // the fused form reduces the first Courant step here
            load_kernel<LAW_HYDRO, ACC64><<<nb, 256, 0, s>>>(aos, c0, c1, m->Uh[r], m->Ul[r], m->Pf, m->GF, m->pp, st,
                                                             m->fused ? m->dcfl : nullptr);
            break;
        case MARA_LAW_MHD:
            load_kernel<LAW_MHD, ACC64><<<nb, 256, 0, s>>>(aos, c0, c1, m->Uh[r], m->Ul[r], m->Pf, m->GF, m->pp, st,
                                                           nullptr);
            break;
        default:
            load_kernel<LAW_RMHD, ACC64><<<nb, 256, 0, s>>>(aos, c0, c1, m->Uh[r], m->Ul[r], m->Pf, m->GF, m->pp, st,
                                                            nullptr);
            break;
    }
}

void mixed_load_aos_range(MixedState* m, const double* aos, long long c0, long long c1, DevStatus* st, cudaStream_t s)
{
    if (c1 <= c0) return;
    if (m->acc64) load_range<true>(m, aos, c0, c1, st, s);
    else load_range<false>(m, aos, c0, c1, st, s);
}

void mixed_load_finish(MixedState* m, DevStatus* st, cudaStream_t s)
{
    // Courant step of the loaded state (the general form reads the FP32
    // primitives), published by mixed_enqueue_courant
    if (!m->fused) courant_general(m, st, s);
}

template <bool ACC64>
static void store_range(MixedState* m, double* aos, long long c0, long long c1, cudaStream_t s)
{
    const unsigned nb = (unsigned) ((c1 - c0 + 255) / 256);
    const int r = host_rot(m);
    switch (m->cfg.law) {
        case MARA_LAW_HYDRO:
            store_kernel<LAW_HYDRO, ACC64><<<nb, 256, 0, s>>>(m->Uh[r], m->Ul[r], aos, c0, c1, m->GF, m->pp);
            break;
        case MARA_LAW_MHD:
            store_kernel<LAW_MHD, ACC64><<<nb, 256, 0, s>>>(m->Uh[r], m->Ul[r], aos, c0, c1, m->GF, m->pp);
            break;
        default:
            store_kernel<LAW_RMHD, ACC64><<<nb, 256, 0, s>>>(m->Uh[r], m->Ul[r], aos, c0, c1, m->GF, m->pp);
            break;
    }
}

void mixed_store_aos_range(MixedState* m, double* aos, long long c0, long long c1, cudaStream_t s)
{
    if (c1 <= c0) return;
    if (m->acc64) store_range<true>(m, aos, c0, c1, s);
    else store_range<false>(m, aos, c0, c1, s);
}

// ---- diagnostics ---------------------------------------------------------------
// interior zone (i, j, k) of the FP32-pair state, converted to FP64
// primitives exactly as a download converts it
template <int LAW, bool ACC64>
struct MixedSrc {
    const float* Uh;
    const float* Ul;
    long long sU;
    int n0, n1;
    double gm1;
    PhysParams pp;
    __device__ __forceinline__ int load(int i, int j, int k, double* P) const
    {
        constexpr int NQ = LawInfo<LAW>::NQ;
        const long long u = ((long long) k * n1 + j) * n0 + i;
        double U[NQ];
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
            if constexpr (ACC64) U[q] = reinterpret_cast<const double*>(Uh)[q * sU + u];
            else U[q] = f2d_exact(Uh[q * sU + u]) + f2d_exact(Ul[q * sU + u]);
        }
        if constexpr (LAW == LAW_HYDRO) {
            hydro_u2p_d(U, gm1, P);
            return ST_OK;
        } else {
            int code = 0;
            const int e = law_cons<LAW>(pp, U, P, &code);
            return e == ST_OK ? ST_OK : (code != 0 ? code : e);
        }
    }
};

template <int LAW, bool ACC64>
static void volume_diag_mixed(MixedState* m, double* partial, int* err, double* out, cudaStream_t s)
{
    const int r = host_rot(m);
    const MixedSrc<LAW, ACC64> src{m->Uh[r], m->Ul[r], m->GF.sU, m->G.n[0], m->G.n[1], m->GF.gm1_d, m->pp};
    const long long zones = (long long) m->G.n[0] * m->G.n[1] * m->G.n[2];
    const long long want = (zones + 255) / 256;
    const int nb = (int) (want < DIAG_BLOCKS ? want : DIAG_BLOCKS);
    k_volume_diag<LAW><<<nb, 256, 0, s>>>(src, m->pp, m->G.n[0], m->G.n[1], zones, m->G.dV, partial, err);
    k_diag_final<<<1, 32, 0, s>>>(partial, nb, DiagInfo<LAW>::ND, out);
}

void mixed_volume_diagnostics(MixedState* m, double* partial, int* err, double* out, cudaStream_t s)
{
    if (m->acc64) {
        switch (m->cfg.law) {
            case MARA_LAW_HYDRO: volume_diag_mixed<LAW_HYDRO, true>(m, partial, err, out, s); break;
            case MARA_LAW_MHD: volume_diag_mixed<LAW_MHD, true>(m, partial, err, out, s); break;
            default: volume_diag_mixed<LAW_RMHD, true>(m, partial, err, out, s); break;
        }
        return;
    }
    switch (m->cfg.law) {
        case MARA_LAW_HYDRO: volume_diag_mixed<LAW_HYDRO, false>(m, partial, err, out, s); break;
        case MARA_LAW_MHD: volume_diag_mixed<LAW_MHD, false>(m, partial, err, out, s); break;
        default: volume_diag_mixed<LAW_RMHD, false>(m, partial, err, out, s); break;
    }
}

// ---- general form ------------------------------------------------------------
// a launch in the general form's chain of programmatic dependents (pdl_chain)
template <typename... KArgs, typename... Args>
static void chain_launch(void (*kernel)(KArgs...), dim3 grid, dim3 block, cudaStream_t s, Args&&... args)
{
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t lc = {};
    lc.gridDim = grid;
    lc.blockDim = block;
    lc.stream = s;
    lc.attrs = at;
    lc.numAttrs = 1;
    cudaLaunchKernelEx(&lc, kernel, std::forward<Args>(args)...);
}

template <int LAW, int RECON, int RIEMANN>
static void flux_f_launch(MixedState* m, int axis, const int* done, DevStatus* st, cudaStream_t s)
{
    const GridF& G = m->GF;
    int lo[3], nb[3];
    for (int a = 0; a < 3; ++a) {
        if (a == axis) { lo[a] = G.g[a]; nb[a] = G.n[a] + 1; }
        else if (G.n[a] > 1) { const int e = G.ct ? 1 : 0; lo[a] = G.g[a] - e; nb[a] = G.n[a] + 2 * e; }
        else { lo[a] = 0; nb[a] = 1; }
    }
    dim3 grid((unsigned) (((long long) nb[0] * nb[1] + 127) / 128), nb[2]);
#define MARA_FLUX_ARGS m->Pf, m->F[axis], G, axis, lo[0], lo[1], lo[2], nb[0], nb[1], done, st
    // hydro and MHD fluxes take the axis at compile time; the relativistic
    // law's cost is its quartic, so it keeps one kernel for all axes
    if constexpr (LAW == LAW_RMHD) {
        chain_launch(flux_f_kernel<LAW, RECON, RIEMANN, -1>, grid, dim3(128), s, MARA_FLUX_ARGS);
    } else {
        switch (axis) {
            case 0: chain_launch(flux_f_kernel<LAW, RECON, RIEMANN, 0>, grid, dim3(128), s, MARA_FLUX_ARGS); break;
            case 1: chain_launch(flux_f_kernel<LAW, RECON, RIEMANN, 1>, grid, dim3(128), s, MARA_FLUX_ARGS); break;
            default: chain_launch(flux_f_kernel<LAW, RECON, RIEMANN, 2>, grid, dim3(128), s, MARA_FLUX_ARGS); break;
        }
    }
#undef MARA_FLUX_ARGS
}

template <int LAW, int RECON>
static void flux_f_r(MixedState* m, int axis, const int* done, DevStatus* st, cudaStream_t s)
{
    if (m->cfg.riemann == MARA_RIEMANN_HLLC) flux_f_launch<LAW, RECON, RIEMANN_HLLC>(m, axis, done, st, s);
    else flux_f_launch<LAW, RECON, RIEMANN_HLLE>(m, axis, done, st, s);
}

template <int LAW>
static void flux_f(MixedState* m, int axis, const int* done, DevStatus* st, cudaStream_t s)
{
    switch (m->cfg.recon) {
        case MARA_RECON_PCM: flux_f_r<LAW, RECON_PCM>(m, axis, done, st, s); break;
        case MARA_RECON_PLM: flux_f_r<LAW, RECON_PLM>(m, axis, done, st, s); break;
        default: flux_f_r<LAW, RECON_WENO5>(m, axis, done, st, s); break;
    }
}

static const float B_TAB[3][3] = {{1.f, 0.f, 0.f}, {1.f, 0.5f, 0.f}, {1.f, 0.25f, 2.f / 3.f}};


static void general_step(MixedState* m, const double* dt, DevStatus* st, cudaStream_t s)
{
    const int order = m->cfg.rk_order;
    const int* done = &st->done;
    FluxViewF V;
    for (int a = 0; a < 3; ++a) V.F[a] = m->F[a];
    for (int e = 0; e < 3; ++e) V.E[e] = m->E[e];
    V.sF = m->G.sF;
    V.M0 = m->G.N[0] + 1;
    V.M1 = m->G.N[1] + 1;
    const int sb = 0, tb = 1;
    for (int rk = 0; rk < order; ++rk) {
        for (int a = 0; a < 3; ++a) {
            if (m->G.n[a] <= 1) continue;
            timed(m, s, [&] {
                switch (m->cfg.law) {
                    case MARA_LAW_HYDRO: flux_f<LAW_HYDRO>(m, a, done, st, s); break;
                    case MARA_LAW_MHD: flux_f<LAW_MHD>(m, a, done, st, s); break;
                    default: flux_f<LAW_RMHD>(m, a, done, st, s); break;
                }
            });
        }
        if (m->E[0]) {
            dim3 eg((unsigned) (((long long) V.M0 * V.M1 + 127) / 128), m->G.N[2] + 1);
            timed(m, s, [&] {
                chain_launch(ct_emf_kernel, eg, dim3(128), s, V, m->E[0], m->E[1], m->E[2], V.M0, V.M1,
                             m->G.N[2] + 1, (int) (m->G.n[0] > 1), (int) (m->G.n[1] > 1), (int) (m->G.n[2] > 1));
            });
        }
        const float b = B_TAB[order - 1][rk];
        const int src = rk == 0 ? sb : tb;
        const int dst = rk == order - 1 ? sb : tb;
        const bool last = rk == order - 1;
        // the last stage also reduces the new state's Courant step
        if (last) chain_launch(k_cfl_reset, dim3(1), dim3(1), s, m->dcfl_next);
        unsigned long long* cfl = last ? m->dcfl_next : nullptr;
        dim3 grid((m->G.n[0] + 127) / 128, m->G.n[1], m->G.n[2]);
        timed(m, s, [&] {
#define MARA_UPDATE_ARGS m->Pf, m->Uh[sb], m->Ul[sb], m->Uh[src], m->Ul[src], m->Uh[dst], m->Ul[dst], V, m->GF, dt, b, 1.f - b, done, st, cfl
            if (m->acc64) {
                switch (m->cfg.law) {
                    case MARA_LAW_HYDRO: chain_launch(update_f_kernel<LAW_HYDRO, true>, grid, dim3(128), s, MARA_UPDATE_ARGS); break;
                    case MARA_LAW_MHD: chain_launch(update_f_kernel<LAW_MHD, true>, grid, dim3(128), s, MARA_UPDATE_ARGS); break;
                    default: chain_launch(update_f_kernel<LAW_RMHD, true>, grid, dim3(128), s, MARA_UPDATE_ARGS); break;
                }
            } else {
                switch (m->cfg.law) {
                    case MARA_LAW_HYDRO: chain_launch(update_f_kernel<LAW_HYDRO, false>, grid, dim3(128), s, MARA_UPDATE_ARGS); break;
                    case MARA_LAW_MHD: chain_launch(update_f_kernel<LAW_MHD, false>, grid, dim3(128), s, MARA_UPDATE_ARGS); break;
                    default: chain_launch(update_f_kernel<LAW_RMHD, false>, grid, dim3(128), s, MARA_UPDATE_ARGS); break;
                }
            }
#undef MARA_UPDATE_ARGS
        });
    }
    chain_launch(k_cfl_commit, dim3(1), dim3(1), s, m->dcfl, (const unsigned long long*) m->dcfl_next,
                 (const DevStatus*) st);
}

// ---- fused hydro tiles ------------------------------------------------------
template <int DIM, int RECON, int RIEMANN>
static void tile_launch(MixedState* m, const double* dt, DevStatus* st, cudaStream_t s, int stage, float b, int last)
{
    constexpr int TX = DIM == 2 ? 32 : 256, TY = DIM == 2 ? 16 : 1, NT = 256;
    // the first stage follows the step-start kernel as its programmatic
    // dependent (an eager timing pass launches it plainly)
    const int after_begin = stage == 0 && !m->timing;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3((unsigned) m->ctas);
    lc.blockDim = dim3(NT);
    lc.stream = s;
    lc.attrs = at;
    lc.numAttrs = after_begin ? 1 : 0;
    if (m->acc64)
        cudaLaunchKernelEx(&lc, hydro_tile_kernel<DIM, RECON, RIEMANN, TX, TY, NT, true>, (const HGrid*) m->dgrid,
                           (const TileRef*) m->dtiles, (const int*) m->dntiles, (const int*) m->drot, dt, 0,
                           (const int*) &st->done, 0, stage, b, 1.f - b, last, m->dcfl, 0, after_begin);
    else
        cudaLaunchKernelEx(&lc, hydro_tile_kernel<DIM, RECON, RIEMANN, TX, TY, NT, false>, (const HGrid*) m->dgrid,
                           (const TileRef*) m->dtiles, (const int*) m->dntiles, (const int*) m->drot, dt, 0,
                           (const int*) &st->done, 0, stage, b, 1.f - b, last, m->dcfl, 0, after_begin);
}

template <int DIM>
static void tile_dispatch(MixedState* m, const double* dt, DevStatus* st, cudaStream_t s, int stage, float b, int last)
{
    const bool hllc = m->cfg.riemann == MARA_RIEMANN_HLLC;
    if (m->cfg.recon == MARA_RECON_PCM) {
        if (hllc) tile_launch<DIM, RECON_PCM, RIEMANN_HLLC>(m, dt, st, s, stage, b, last);
        else tile_launch<DIM, RECON_PCM, RIEMANN_HLLE>(m, dt, st, s, stage, b, last);
    } else {
        if (hllc) tile_launch<DIM, RECON_PLM, RIEMANN_HLLC>(m, dt, st, s, stage, b, last);
        else tile_launch<DIM, RECON_PLM, RIEMANN_HLLE>(m, dt, st, s, stage, b, last);
    }
}

// the stages of one step; the Courant reduction slot has been reset
static void fused_step(MixedState* m, const double* dt, DevStatus* st, cudaStream_t s)
{
    const int order = m->cfg.rk_order;
    for (int rk = 0; rk < order; ++rk) {
        const int last = rk == order - 1;
        const float b = B_TAB[order - 1][rk];
        timed(m, s, [&] {
            if (m->G.n[1] > 1) tile_dispatch<2>(m, dt, st, s, rk, b, last);
            else tile_dispatch<1>(m, dt, st, s, rk, b, last);
        });
    }
    if (order == 1) k_rot_flip<<<1, 1, 0, s>>>(m->drot, st);
}

void mixed_enqueue_step(MixedState* m, const double* dt, DevStatus* st, cudaStream_t s, int64_t*)
{
    if (m->fused) {
        k_cfl_reset<<<1, 1, 0, s>>>(m->dcfl);
        fused_step(m, dt, st, s);
    } else {
        general_step(m, dt, st, s);
    }
    if (m->fused && m->cfg.rk_order == 1) m->rot ^= 1;
}

bool mixed_enqueue_run_step(MixedState* m, double cfl, double t_final, DevStatus* st, cudaStream_t s)
{
    if (!m->fused) return false;
    k_fused_run_begin<<<1, 1, 0, s>>>(m->dcfl, st, cfl, t_final);
    fused_step(m, &st->dt, st, s);
    if (m->cfg.rk_order == 1) m->rot ^= 1;
    return true;
}

bool mixed_enqueue_advance(MixedState* m, double dt, DevStatus* st, cudaStream_t s)
{
    if (!m->fused) return false;
    k_fused_advance_begin<<<1, 1, 0, s>>>(m->dcfl, st, dt);
    fused_step(m, &st->dt, st, s);
    if (m->cfg.rk_order == 1) m->rot ^= 1;
    return true;
}

// ---- the host step: transfers and stages in one pipelined launch ----------------
// MethodOfLinesTVD::advance on a page-locked host MeshData::P (FP64 AoS, i
// the slowest index: a host row is one column of zones) as one launch whose
// CTAs take items from two ordered queues:
//   IN     one interior host row -> FP32-pair state (read over the chip-to-chip link);
//   WORK   STAGE: one RK stage of one 32 x 16 tile, or
//          OUT: one host row (interior or guard) <- FP32-pair state (written over the link).
// A stage-0 tile needs the IN rows its stencil reads, a later stage the
// previous stage of the 3 x 3 tiles around it, an OUT row the last stage of
// its tile column (a guard row: of the first and the last column).  The
// first in_ctas CTAs take IN rows (they never wait) and then join the
// others, which take WORK items in queue order and wait for the completion
// flags of what each needs.  The WORK queue lists every item after all it
// needs, so the earliest unfinished WORK item has its inputs complete or
// being loaded, and every wait ends.  Both queues take the tile columns in
// transfer order (with periodic boundaries the last column first: it is the
// first one's left neighbour), so transfers in, stages and transfers out
// overlap.  CTAs read the state that other CTAs wrote from L2
// (ld.global.cg).  The per-zone arithmetic is that of load_kernel,
// hydro_tile_kernel and store_kernel.
enum { HS_IN = 0, HS_STAGE = 1, HS_OUT = 4 };  // item kinds: IN, stages 0..2, OUT
constexpr int HS_SLAB = 512;               // cells staged in shared memory at a time
constexpr int HS_POLLS = 1 << 22;          // about a second of waiting, then an error
constexpr int HS_LAG = 256;                // WORK items listed between a stage tile and its readers

__host__ __device__ constexpr int hs_item(int kind, int idx) { return (kind << 26) | idx; }

struct HostStepJob {
    const HGrid* grid;
    double* host;            // device address of the page-locked host array
    const int* in_q;         // IN rows in transfer order
    const int* work_q;       // WORK items (hs_item codes)
    int n_in, n_work;
    int in_ctas;
    int* head;               // [0] IN, [1] WORK, [2] error; zero at launch
    int* in_flag;            // per interior host row, the epoch once loaded
    int* tile_flag;          // per stage and tile, the epoch once written
    DevStatus* st;
    const TileRef* tiles;    // row-major: t = ty * ntx + tx
    int ntx, nty;            // tiles per row / column
    int n0, g0, halo;        // interior and guard host rows, stencil half-width
    long long row;           // cells per host row
    int periodic;
    int r, order;            // the state's buffer, RK order
    float bst[3];
    double dt;
    unsigned long long* cfl;
    int epoch;
    GridF G;
};

// the interior row / tile a stencil coordinate reads (periodic wrap), or -1
__device__ __forceinline__ int hs_wrap(int x, int n, int periodic)
{
    if (x >= 0 && x < n) return x;
    if (periodic) return (x + n) % n;
    return -1;
}

// wait until flag *f holds the epoch (bounded; a timeout sets the error,
// which ends every wait and the launch)
__device__ __forceinline__ void hs_wait_flag(const HostStepJob& J, const int* f)
{
    int polls = 0;
    while (*(volatile const int*) f != J.epoch) {
        if (*(volatile int*) &J.head[2]) return;
        if (++polls > HS_POLLS) {
            if (atomicExch(&J.head[2], 1) == 0) atomicCAS(&J.st->code, 0, MARA_ERR_CUDA);
            return;
        }
        __nanosleep(polls < 32 ? 64 : 512);
    }
}

// one warp: wait for every input of WORK item (kind, idx)
__device__ __forceinline__ void hs_wait_inputs(const HostStepJob& J, int kind, int idx)
{
    const int lane = threadIdx.x & 31;
    if (kind == HS_STAGE) {
        const int tx = idx % J.ntx;
        const int x0 = tx * 32 - J.halo, w = min(32, J.n0 - tx * 32) + 2 * J.halo;
        for (int i = lane; i < w; i += 32) {
            const int x = hs_wrap(x0 + i, J.n0, J.periodic);
            if (x >= 0) hs_wait_flag(J, &J.in_flag[x]);
        }
    } else if (kind < HS_OUT) {
        const int tx = idx % J.ntx, ty = idx / J.ntx;
        const int* f = J.tile_flag + (kind - HS_STAGE - 1) * J.ntx * J.nty;
        if (lane < 9) {
            const int x = hs_wrap(tx + lane % 3 - 1, J.ntx, J.periodic);
            const int y = hs_wrap(ty + lane / 3 - 1, J.nty, J.periodic);
            if (x >= 0 && y >= 0) hs_wait_flag(J, &f[y * J.ntx + x]);
        }
    } else {
        const int* f = J.tile_flag + (J.order - 1) * J.ntx * J.nty;
        const int cols = idx < J.n0 ? 1 : 2;  // a guard row: the first and the last column
        for (int i = lane; i < cols * J.nty; i += 32) {
            const int tx = idx < J.n0 ? idx / 32 : (i < J.nty ? 0 : J.ntx - 1);
            hs_wait_flag(J, &f[(i % J.nty) * J.ntx + tx]);
        }
    }
    __syncwarp();
}

template <int RECON, int RIEMANN>
__global__ void __launch_bounds__(256, 4) host_step_kernel(const __grid_constant__ HostStepJob J)
{
    union Smem {
        TileSmem<2, RECON, 32, 16> t;
        double slab[HS_SLAB * 5];
    };
    __shared__ Smem sm;
    __shared__ int got_k, got_idx;
    const HGrid& g = *J.grid;
    // CTAs 0 .. in_ctas - 1 load, one per SM (a cooperative launch: every CTA
    // is resident, so a WORK item's IN rows are always being taken); thread 0's
    bool in_role = blockIdx.x < J.in_ctas;
    for (;;) {
        __syncthreads();  // the previous item's shared data is consumed
        // 1. the next IN row (the first in_ctas CTAs, while rows are left),
        //    else the next WORK item and, for warp 0, the wait for its inputs
        if (threadIdx.x < 32) {
            int k = -2, idx = 0;
            if (threadIdx.x == 0) {
                if (in_role) {
                    const int h = atomicAdd(&J.head[0], 1);
                    if (h < J.n_in) { k = HS_IN; idx = J.in_q[h]; }
                    else in_role = false;
                }
                if (!in_role) {
                    const int h = atomicAdd(&J.head[1], 1);
                    if (h < J.n_work) { const int c = J.work_q[h]; k = c >> 26; idx = c & ((1 << 26) - 1); }
                }
            }
            k = __shfl_sync(0xffffffffu, k, 0);
            idx = __shfl_sync(0xffffffffu, idx, 0);
            if (k > HS_IN) hs_wait_inputs(J, k, idx);
            __threadfence();
            if (threadIdx.x == 0) { got_k = k; got_idx = idx; }
        }
        __syncthreads();
        const int kind = got_k, idx = got_idx;
        if (kind < 0) return;
        // 2. the work
        if (kind >= HS_STAGE && kind < HS_OUT) {
            const int stage = kind - HS_STAGE;
            const int last = stage == J.order - 1;
            const float b = J.bst[stage];
            struct {
                const HostStepJob* j;
                __device__ float dt() const { return (float) j->dt; }
                __device__ bool proceed() const { return true; }
                __device__ unsigned long long* cfl() const { return j->cfl; }
            } at{&J};
            tile_stage<2, RECON, RIEMANN, 32, 16, 256, true>(sm.t, g, J.tiles[idx], J.r, stage, b, 1.f - b, last, at);
        } else {
            // host row i: interior row idx, or a guard row after the interior ones
            const int i = kind == HS_IN || idx < J.n0 ? J.g0 + idx
                          : idx < J.n0 + J.g0 ? idx - J.n0 : J.g0 + J.n0 + (idx - J.n0 - J.g0);
            const long long c0 = (long long) i * J.row, c1 = c0 + J.row;
            const int out_buf = J.order == 1 ? J.r ^ 1 : J.r;
            for (long long b0 = c0; b0 < c1; b0 += HS_SLAB) {
                const int nc = (int) min((long long) HS_SLAB, c1 - b0);
                if (kind == HS_IN) {
                    // every load in flight before the first use
                    constexpr int PER = HS_SLAB * 5 / 256;
                    double v[PER];
#pragma unroll
                    for (int u = 0; u < PER; ++u) {
                        const int e = threadIdx.x + u * 256;
                        v[u] = e < nc * 5 ? J.host[b0 * 5 + e] : 0.0;
                    }
#pragma unroll
                    for (int u = 0; u < PER; ++u) sm.slab[threadIdx.x + u * 256] = v[u];
                    __syncthreads();
                    const GridF& G = J.G;
                    for (int cc = threadIdx.x; cc < nc; cc += 256) {
                        const int jj = (int) ((b0 + cc) % G.N[1]) - G.g[1];
                        if (jj < 0 || jj >= G.n[1]) continue;
                        double P[5], U[5];
#pragma unroll
                        for (int q = 0; q < 5; ++q) P[q] = sm.slab[cc * 5 + q];
                        hydro_p2u_d(P, G.inv_gm1_d, U);
                        const long long u = (long long) jj * G.n[0] + idx;
#pragma unroll
                        for (int q = 0; q < 5; ++q) {
                            const df d = df_from_double(U[q]);
                            g.Uh[J.r][q * G.sU + u] = d.hi;
                            g.Ul[J.r][q * G.sU + u] = d.lo;
                        }
                    }
                } else {
                    for (int cc = threadIdx.x; cc < nc; cc += 256)
                        store_cell<LAW_HYDRO, true>(g.Uh[out_buf], g.Ul[out_buf], b0 + cc, J.G, PhysParams(),
                                                    &sm.slab[cc * 5]);
                    __syncthreads();
                    for (int e = threadIdx.x; e < nc * 5; e += 256) J.host[b0 * 5 + e] = sm.slab[e];
                }
                __syncthreads();
            }
        }
        // 3. publish
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            if (kind == HS_IN) *(volatile int*) &J.in_flag[idx] = J.epoch;
            else if (kind < HS_OUT) *(volatile int*) &J.tile_flag[(kind - HS_STAGE) * J.ntx * J.nty + idx] = J.epoch;
        }
    }
}

__global__ void k_host_step_begin(DevStatus* st, unsigned long long* cfl, int* head, int* drot, int rot_after,
                                  double dt)
{
    st->dt = dt;
    *cfl = (unsigned long long) __double_as_longlong(DBL_MAX);
    for (int k = 0; k < 8; ++k) head[k] = 0;
    *drot = rot_after;
}

struct HostStep {
    int ntx = 0, nty = 0;
    int* dq = nullptr;        // the IN queue, then the WORK queue
    int n_in = 0, n_work = 0;
    int* dhead = nullptr;
    int* dflags = nullptr;    // IN row flags, then the stages' tile flags
    size_t nflags = 0;
    int epoch = 0;
    int grid = 0;             // CTAs of the launch
    int in_ctas = 0;
};

static void host_step_destroy(HostStep* hs)
{
    if (!hs) return;
    cudaFree(hs->dq);
    cudaFree(hs->dhead);
    cudaFree(hs->dflags);
    delete hs;
}

bool mixed_host_step_capable(const MixedState* m)
{
    // a stage reads one tile either side only if the last tile row and column
    // hold at least the two-zone halo; below about half a million zones the
    // pipeline's fixed costs outweigh the overlap (256^2: 0.098 ms against
    // 0.085 ms unpipelined; 512^2 even; 1024^2 0.45 against 0.56 ms)
    const int rx = m->G.n[0] % 32, ry = m->G.n[1] % 16;
    return m->fused && !m->acc64 && m->G.n[1] > 1 && m->G.N[2] == 1 && m->G.n[0] >= 128 && m->tx == 32 && m->ty == 16 &&
           (rx == 0 || rx >= 2) && (ry == 0 || ry >= 2) && (long long) m->G.n[0] * m->G.n[1] >= (1 << 19) &&
           !m->hs_unavailable;
}

template <int RECON, int RIEMANN>
static int host_step_occupancy()
{
    int per = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, host_step_kernel<RECON, RIEMANN>, 256, 0) != cudaSuccess)
        return 0;
    return per;
}

// The queues.  Tile columns in transfer order; IN lists their rows; WORK
// lists, after each column's rows, every stage tile whose inputs are now
// listed, stage by stage, then the OUT rows of every column whose last stage
// is; the guard rows come last.  A stage tile or an OUT row is listed only
// HS_LAG items after the stage tiles it reads, so that they are usually
// complete when a CTA takes it (a CTA waiting for inputs holds its slot);
// when nothing else can be listed the lag is dropped.
static void host_step_queues(int n0, int ntx, int nty, int order, bool periodic, int g0, std::vector<int>& in_q,
                             std::vector<int>& work_q)
{
    std::vector<char> in(ntx, 0), out(ntx, 0);
    // per stage and tile: -1 until listed, then its WORK position
    std::vector<std::vector<int>> st(order, std::vector<int>((size_t) ntx * nty, -1));
    std::vector<int> last_pos(ntx, -1), cnt_last(ntx, 0);
    auto wrap = [&](int x, int n, bool& ok) {
        ok = true;
        if (x >= 0 && x < n) return x;
        if (periodic) return (x + n) % n;
        ok = false;
        return 0;
    };
    // list everything whose inputs were listed at least `lag` items before
    auto sweep = [&](int lag) {
        bool any = false;
        for (bool more = true; more;) {
            more = false;
            const int now = (int) work_q.size();
            for (int k = 0; k < order; ++k)
                for (int tx = 0; tx < ntx; ++tx)
                    for (int ty = 0; ty < nty; ++ty) {
                        const int t = ty * ntx + tx;
                        if (st[k][t] >= 0) continue;
                        bool ready = true;
                        if (k == 0) {
                            for (int d = -1; d <= 1 && ready; ++d) {
                                bool ok;
                                const int x = wrap(tx + d, ntx, ok);
                                if (ok) ready = in[x];
                            }
                        } else {
                            for (int dy = -1; dy <= 1 && ready; ++dy)
                                for (int dx = -1; dx <= 1 && ready; ++dx) {
                                    bool okx, oky;
                                    const int x = wrap(tx + dx, ntx, okx), y = wrap(ty + dy, nty, oky);
                                    if (okx && oky) {
                                        const int p = st[k - 1][y * ntx + x];
                                        ready = p >= 0 && p + lag <= now;
                                    }
                                }
                        }
                        if (!ready) continue;
                        st[k][t] = (int) work_q.size();
                        work_q.push_back(hs_item(HS_STAGE + k, t));
                        if (k == order - 1) {
                            cnt_last[tx]++;
                            last_pos[tx] = st[k][t];
                        }
                        more = any = true;
                    }
            for (int tx = 0; tx < ntx; ++tx)
                if (!out[tx] && cnt_last[tx] == nty && last_pos[tx] + lag <= now) {
                    for (int x = tx * 32; x < std::min(n0, tx * 32 + 32); ++x) work_q.push_back(hs_item(HS_OUT, x));
                    out[tx] = 1;
                    more = any = true;
                }
        }
        return any;
    };
    std::vector<int> cols;
    if (periodic) cols.push_back(ntx - 1);
    for (int b = 0; b < ntx; ++b) if (!(periodic && b == ntx - 1)) cols.push_back(b);
    for (int b : cols) {
        for (int x = b * 32; x < std::min(n0, b * 32 + 32); ++x) in_q.push_back(x);
        in[b] = 1;
        sweep(HS_LAG);
    }
    while (sweep(HS_LAG) || sweep(0)) {
    }
    for (int k = 0; k < 2 * g0; ++k) work_q.push_back(hs_item(HS_OUT, n0 + k));
}

static int host_step_setup(MixedState* m)
{
    HostStep* hs = new HostStep();
    m->hs = hs;
    const int order = m->cfg.rk_order;
    hs->ntx = (m->G.n[0] + 31) / 32;
    hs->nty = (m->G.n[1] + 15) / 16;
    std::vector<int> in_q, work_q;
    host_step_queues(m->G.n[0], hs->ntx, hs->nty, order, m->G.bc == BC_PERIODIC, m->G.g[0], in_q, work_q);
    hs->n_in = (int) in_q.size();
    hs->n_work = (int) work_q.size();
    std::vector<int> all(in_q);
    all.insert(all.end(), work_q.begin(), work_q.end());
    hs->nflags = (size_t) m->G.n[0] + (size_t) order * hs->ntx * hs->nty;
    if (cudaMalloc((void**) &hs->dq, sizeof(int) * all.size()) != cudaSuccess ||
        cudaMalloc((void**) &hs->dhead, sizeof(int) * 8) != cudaSuccess ||
        cudaMalloc((void**) &hs->dflags, sizeof(int) * hs->nflags) != cudaSuccess)
        return MARA_ERR_CUDA;
    if (cudaMemcpy(hs->dq, all.data(), sizeof(int) * all.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(hs->dflags, 0, sizeof(int) * hs->nflags) != cudaSuccess)
        return MARA_ERR_CUDA;
    int per = 0, dev = 0, sms = 0;
    const bool hllc = m->cfg.riemann == MARA_RIEMANN_HLLC;
    if (m->cfg.recon == MARA_RECON_PCM)
        per = hllc ? host_step_occupancy<RECON_PCM, RIEMANN_HLLC>() : host_step_occupancy<RECON_PCM, RIEMANN_HLLE>();
    else
        per = hllc ? host_step_occupancy<RECON_PLM, RIEMANN_HLLC>() : host_step_occupancy<RECON_PLM, RIEMANN_HLLE>();
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (per < 2) return MARA_ERR_CUDA;
    hs->grid = per * sms;
    hs->in_ctas = sms;  // one loading CTA per SM keeps the link busy
    return MARA_OK;
}

template <int RECON, int RIEMANN>
static cudaError_t host_step_launch(const HostStepJob& J, int grid, cudaStream_t s)
{
    void* args[] = {(void*) &J};
    return cudaLaunchCooperativeKernel((const void*) host_step_kernel<RECON, RIEMANN>, dim3(grid), dim3(256), args, 0,
                                       s);
}

int mixed_advance_host_step(MixedState* m, double* host_dev, double dt, DevStatus* st, cudaStream_t s,
                            int64_t* launches)
{
    if (m->hs_unavailable) return MIXED_NOT_TAKEN;
    if (!m->hs) {
        if (host_step_setup(m)) {
            host_step_destroy(m->hs);
            m->hs = nullptr;
            m->hs_unavailable = true;
            cudaGetLastError();
            return MIXED_NOT_TAKEN;
        }
    }
    HostStep* hs = m->hs;
    const int order = m->cfg.rk_order;
    const int r = host_rot(m);
    const int rot_after = order == 1 ? r ^ 1 : r;
    hs->epoch = hs->epoch == 0x3fffffff ? 1 : hs->epoch + 1;
    if (hs->epoch == 1) cudaMemsetAsync(hs->dflags, 0, sizeof(int) * hs->nflags, s);
    k_host_step_begin<<<1, 1, 0, s>>>(st, m->dcfl, hs->dhead, m->drot, rot_after, dt);
    HostStepJob J = {};
    J.grid = m->dgrid;
    J.host = host_dev;
    J.in_q = hs->dq;
    J.work_q = hs->dq + hs->n_in;
    J.n_in = hs->n_in;
    J.n_work = hs->n_work;
    J.in_ctas = hs->in_ctas;
    J.head = hs->dhead;
    J.in_flag = hs->dflags;
    J.tile_flag = hs->dflags + m->G.n[0];
    J.st = st;
    J.tiles = m->dtiles;
    J.ntx = hs->ntx;
    J.nty = hs->nty;
    J.n0 = m->G.n[0];
    J.g0 = m->G.g[0];
    J.halo = m->cfg.recon == MARA_RECON_PCM ? 1 : 2;
    J.row = (long long) m->G.N[1] * m->G.N[2];
    J.periodic = m->G.bc == BC_PERIODIC;
    J.r = r;
    J.order = order;
    for (int k = 0; k < 3; ++k) J.bst[k] = B_TAB[order - 1][k];
    J.dt = dt;
    J.cfl = m->dcfl;
    J.epoch = hs->epoch;
    J.G = m->GF;
    cudaError_t e;
    const bool hllc = m->cfg.riemann == MARA_RIEMANN_HLLC;
    if (m->cfg.recon == MARA_RECON_PCM)
        e = hllc ? host_step_launch<RECON_PCM, RIEMANN_HLLC>(J, hs->grid, s)
                 : host_step_launch<RECON_PCM, RIEMANN_HLLE>(J, hs->grid, s);
    else
        e = hllc ? host_step_launch<RECON_PLM, RIEMANN_HLLC>(J, hs->grid, s)
                 : host_step_launch<RECON_PLM, RIEMANN_HLLE>(J, hs->grid, s);
    if (e != cudaSuccess) {
        // a cooperative launch this device cannot run: the unpipelined path
        cudaGetLastError();
        m->hs_unavailable = true;
        return MIXED_NOT_TAKEN;
    }
    *launches += 2;
    m->rot = rot_after;
    return MARA_OK;
}

int mixed_launches_per_step(const MixedState* m)
{
    // fused: the step-begin kernel, one launch per stage, the RK1 rotation
    if (m->fused) return 1 + m->cfg.rk_order + (m->cfg.rk_order == 1 ? 1 : 0);
    // general: per stage the flux launches, the edge EMFs (flux CT), the
    // update; per step the Courant slot's reset and commit
    int axes = 0;
    for (int a = 0; a < 3; ++a) axes += m->G.n[a] > 1;
    return m->cfg.rk_order * (axes + 1 + (m->E[0] ? 1 : 0)) + 2;
}

void mixed_enqueue_courant(MixedState* m, DevStatus* st, cudaStream_t s) { k_cfl_publish<<<1, 1, 0, s>>>(m->dcfl, st); }
int mixed_parity(const MixedState* m) { return m->rot & 1; }
bool mixed_fused(const MixedState* m) { return m->fused; }

// ---- small 1-D grids: many steps per launch on one thread-block cluster -------
bool mixed_cluster_capable(const MixedState* m)
{
    return m->fused && m->G.n[1] == 1 && m->G.n[2] == 1 &&
           m->G.n[0] <= CLUSTER1D_MAX_CTAS * CLUSTER1D_MAX_ZONES_PER_CTA;
}

template <int RECON, int RIEMANN, bool ACC64>
static int cluster_launch(MixedState* m, int nsteps, double cfl, double t_final, DevStatus* st, cudaStream_t s)
{
    const int n = m->G.n[0];
    // a single grid is latency-bound: up to the wide cluster size where it
    // fits (a step of 8192 zones: 11.9 us on 8 CTAs, 8.5 us on 16)
    int C = cluster1d_ctas(n);
    const int wide = cluster1d_ctas(n, CLUSTER1D_WIDE_CTAS);
    if (wide > C && cluster1d_fits<RECON, RIEMANN, ACC64>(wide, (n + wide - 1) / wide)) C = wide;
    Cluster1DJob job = {};
    job.grids = m->dgrid;
    job.t = &st->t;
    job.steps = &st->steps;
    job.dt = &st->dt;
    job.done = &st->done;
    job.used = &st->dt_bits;
    job.cfl = m->dcfl;
    job.t_final = t_final;
    job.cfl_number = cfl;
    job.done_value = 1;
    job.order = m->cfg.rk_order;
    job.nsteps = nsteps;
    job.buffer = host_rot(m);
    const cudaError_t e = launch_cluster1d<RECON, RIEMANN, ACC64>(job, 1, C, (n + C - 1) / C, s);
    return e == cudaSuccess ? MARA_OK : MARA_ERR_CUDA;
}

int mixed_enqueue_cluster_steps(MixedState* m, int nsteps, double cfl, double t_final, DevStatus* st, cudaStream_t s)
{
    const bool hllc = m->cfg.riemann == MARA_RIEMANN_HLLC;
    if (m->acc64) {
        if (m->cfg.recon == MARA_RECON_PCM)
            return hllc ? cluster_launch<RECON_PCM, RIEMANN_HLLC, true>(m, nsteps, cfl, t_final, st, s)
                        : cluster_launch<RECON_PCM, RIEMANN_HLLE, true>(m, nsteps, cfl, t_final, st, s);
        return hllc ? cluster_launch<RECON_PLM, RIEMANN_HLLC, true>(m, nsteps, cfl, t_final, st, s)
                    : cluster_launch<RECON_PLM, RIEMANN_HLLE, true>(m, nsteps, cfl, t_final, st, s);
    }
    if (m->cfg.recon == MARA_RECON_PCM)
        return hllc ? cluster_launch<RECON_PCM, RIEMANN_HLLC, false>(m, nsteps, cfl, t_final, st, s)
                    : cluster_launch<RECON_PCM, RIEMANN_HLLE, false>(m, nsteps, cfl, t_final, st, s);
    return hllc ? cluster_launch<RECON_PLM, RIEMANN_HLLC, false>(m, nsteps, cfl, t_final, st, s)
                : cluster_launch<RECON_PLM, RIEMANN_HLLE, false>(m, nsteps, cfl, t_final, st, s);
}
void mixed_set_parity(MixedState* m, int p) { m->rot = p; }
// the state buffer the device rotation holds (the stream is idle): steps
// enqueued after the loop was done did not turn it
void mixed_sync_rotation(MixedState* m, cudaStream_t s)
{
    cudaMemcpyAsync(&m->rot, m->drot, sizeof(int), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
}
void mixed_advance_parity(MixedState* m) { if (m->fused && m->cfg.rk_order == 1) m->rot ^= 1; }
void mixed_set_timing(MixedState* m, int on) { m->timing = on; }
const float* mixed_primitives(const MixedState* m) { return m->Pf; }

void mixed_kernel_times(MixedState* m, double ms[3], int64_t launches[3])
{
    for (auto& e : m->ev) {
        float t = 0.f;
        cudaEventSynchronize(e.second);
        cudaEventElapsedTime(&t, e.first, e.second);
        ms[0] += t;
        launches[0] += 1;
        cudaEventDestroy(e.first);
        cudaEventDestroy(e.second);
    }
    m->ev.clear();
}

} // namespace mara
