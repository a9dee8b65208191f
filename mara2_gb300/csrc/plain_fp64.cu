// plain_fp64.cu -- the plain FP64 path: one face-flux sweep kernel per
// fleshed axis, then one fused update kernel per RK stage, plus the Courant
// reduction.  Compiled with --fmad=false (see mara2_gb300/build.py) so that
// the arithmetic rounds as the reference's CPU build does.
//
// Per stage (MethodOfLinesTVD::advance, SolutionSchemes.cpp:191-274):
//   flux_kernel<axis>   MeshOperator::godunov (MeshOperator.cpp:443-525):
//                       gather the 2s-cell stencil along the axis, intercell
//                       flux (reconstruction + fromPrimitive x2 + Riemann),
//                       raw flux stored per face.  Faces are those the
//                       interior update reads: along the axis the interior
//                       faces, across it the interior rows plus one guard row
//                       on each side when flux CT needs transverse neighbours.
//   update_kernel       per interior zone: CellCenteredFieldCT's flux CT on
//                       the magnetic fluxes of the zone's six faces
//                       (CellCenteredFieldCT.cpp:14-134), the divergence
//                       (MeshOperator.cpp:323-381), the RK combine
//                       (SolutionSchemes.cpp:232-235), fromConserved
//                       (FieldOperator::recoverPrimitive, FieldOperator.cpp:
//                       41-82) and the guard fill: boundary conditions are
//                       copies (periodic, outflow) or mirrored copies
//                       (reflecting) of interior zones applied axis by axis,
//                       so every guard zone equals one interior zone (velocity
//                       components negated on reflecting axes) and the zone
//                       that owns a value writes all of its guard images.
#include "../../include/mara_gpu.h"
#include "internal.h"
#include "physics_fp64.cuh"

namespace mara {

template <int RECON> struct ReconInfo;
template <> struct ReconInfo<RECON_PCM> { static constexpr int S = 1; };
template <> struct ReconInfo<RECON_PLM> { static constexpr int S = 2; };
template <> struct ReconInfo<RECON_WENO5> { static constexpr int S = 3; };

__device__ __forceinline__ void record_status(DevStatus* st, int code)
{
    atomicCAS(&st->code, 0, code);
}

// ---------------------------------------------------------------------------
template <int LAW, int RECON, int RIEMANN>
__global__ void __launch_bounds__(128) flux_kernel(const double* __restrict__ P, double* __restrict__ F,
                                                   GridDesc G, PhysParams pp, int axis,
                                                   int lo0, int lo1, int lo2, int nb0, int nb1,
                                                   DevStatus* __restrict__ st)
{
    constexpr int NQ = LawInfo<LAW>::NQ;
    constexpr int S = ReconInfo<RECON>::S;
    if (st->code != 0 || st->done) return;
    if (st->failures != 0) { st->halt = 1; return; }  // failures are final once the stage ended
    // the faces of one z-slice as one index space (rows of n + 1 or n + 2
    // faces would leave a nearly empty block per row)
    const unsigned lin = blockIdx.x * blockDim.x + threadIdx.x;
    if (lin >= (unsigned) nb0 * (unsigned) nb1) return;
    const int i = lo0 + (int) (lin % (unsigned) nb0), j = lo1 + (int) (lin / (unsigned) nb0), k = lo2 + blockIdx.y;
    const long long stride = axis == 0 ? 1 : axis == 1 ? (long long) G.N[0] : (long long) G.N[0] * G.N[1];
    const long long base = ((long long) k * G.N[1] + j) * G.N[0] + i; // cell on the right of the face
    const double n[3] = {G.nrm[axis][0], G.nrm[axis][1], G.nrm[axis][2]};

    double PL[NQ], PR[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
        double v[2 * S];
#pragma unroll
        for (int c = 0; c < 2 * S; ++c) v[c] = P[q * G.sP + base + (c - S) * stride];
        if constexpr (RECON == RECON_PCM) {
            PL[q] = v[0];
            PR[q] = v[1];
        } else if constexpr (RECON == RECON_PLM) {
            PL[q] = v[1] + +1.0 * 0.5 * minmod(pp.plm_theta, v[0], v[1], v[2]);
            PR[q] = v[2] + -1.0 * 0.5 * minmod(pp.plm_theta, v[1], v[2], v[3]);
        } else {
            PL[q] = weno5<true>(&v[2], pp.weno_is, pp.shenzha_A);
            PR[q] = weno5<false>(&v[3], pp.weno_is, pp.shenzha_A);
        }
    }
    StateD<NQ> L, R;
    int e = law_prim<LAW>(pp, PL, n, L);
    if (e == ST_OK) e = law_prim<LAW>(pp, PR, n, R);
    if (e != ST_OK) { record_status(st, e); return; }
    double Fh[NQ];
    if constexpr (RIEMANN == RIEMANN_HLLC) hllc<NQ>(L, R, n, Fh);
    else hlle<NQ>(L, R, Fh);
    const long long f = ((long long) k * (G.N[1] + 1) + j) * (G.N[0] + 1) + i;
#pragma unroll
    for (int q = 0; q < NQ; ++q) F[q * G.sF + f] = Fh[q];
}

// ---------------------------------------------------------------------------
struct FluxView {
    const double* F[3];
    long long sF;
    int M0, M1; // (N0+1), (N1+1)
    __device__ __forceinline__ double at(int a, int q, int i, int j, int k) const
    {
        return F[a][q * sF + ((long long) k * M1 + j) * M0 + i];
    }
};

// Flux of field q through the face of axis a at flux index (i, j, k), after
// CellCenteredFieldCT::correctGodunovFluxes when ct is on (magnetic index 5).
template <int NQ>
__device__ __forceinline__ double face_flux(const FluxView& V, const GridDesc& G, int a, int q, int i, int j, int k)
{
    if ((NQ == 8 || NQ == 9) && G.ct && q >= 5 && q <= 7) {
        const int B0 = 5, B1 = 6, B2 = 7;
        const bool fx = G.n[0] > 1, fy = G.n[1] > 1, fz = G.n[2] > 1;
        if (a == 0) {
            if (q == B0) return 0.0;
            if (q == B1 && fy)
                return 0.125 * (+2 * V.at(0, B1, i, j, k) + 1 * V.at(0, B1, i, j + 1, k) + 1 * V.at(0, B1, i, j - 1, k)
                                - 1 * V.at(1, B0, i, j + 1, k) - 1 * V.at(1, B0, i - 1, j + 1, k)
                                - 1 * V.at(1, B0, i, j, k) - 1 * V.at(1, B0, i - 1, j, k));
            if (q == B2 && fz)
                return 0.125 * (+2 * V.at(0, B2, i, j, k) + 1 * V.at(0, B2, i, j, k + 1) + 1 * V.at(0, B2, i, j, k - 1)
                                - 1 * V.at(2, B0, i, j, k + 1) - 1 * V.at(2, B0, i - 1, j, k + 1)
                                - 1 * V.at(2, B0, i, j, k) - 1 * V.at(2, B0, i - 1, j, k));
        } else if (a == 1) {
            if (q == B1) return 0.0;
            if (q == B2 && fz)
                return 0.125 * (+2 * V.at(1, B2, i, j, k) + 1 * V.at(1, B2, i, j, k + 1) + 1 * V.at(1, B2, i, j, k - 1)
                                - 1 * V.at(2, B1, i, j, k + 1) - 1 * V.at(2, B1, i, j - 1, k + 1)
                                - 1 * V.at(2, B1, i, j, k) - 1 * V.at(2, B1, i, j - 1, k));
            if (q == B0 && fx)
                return 0.125 * (+2 * V.at(1, B0, i, j, k) + 1 * V.at(1, B0, i + 1, j, k) + 1 * V.at(1, B0, i - 1, j, k)
                                - 1 * V.at(0, B1, i + 1, j, k) - 1 * V.at(0, B1, i + 1, j - 1, k)
                                - 1 * V.at(0, B1, i, j, k) - 1 * V.at(0, B1, i, j - 1, k));
        } else {
            if (q == B2) return 0.0;
            if (q == B0 && fx)
                return 0.125 * (+2 * V.at(2, B0, i, j, k) + 1 * V.at(2, B0, i + 1, j, k) + 1 * V.at(2, B0, i - 1, j, k)
                                - 1 * V.at(0, B2, i + 1, j, k) - 1 * V.at(0, B2, i + 1, j, k - 1)
                                - 1 * V.at(0, B2, i, j, k) - 1 * V.at(0, B2, i, j, k - 1));
            if (q == B1 && fy)
                return 0.125 * (+2 * V.at(2, B1, i, j, k) + 1 * V.at(2, B1, i, j + 1, k) + 1 * V.at(2, B1, i, j - 1, k)
                                - 1 * V.at(1, B2, i, j + 1, k) - 1 * V.at(1, B2, i, j + 1, k - 1)
                                - 1 * V.at(1, B2, i, j, k) - 1 * V.at(1, B2, i, j, k - 1));
        }
    }
    return V.at(a, q, i, j, k);
}

// Guard images of interior index ii along one axis: full indices that the
// boundary condition fills with zone ii (first entry: the zone itself).
// Returns the count; flip[m] marks reflected images.
template <int LAW>
__global__ void __launch_bounds__(128) update_kernel(const double* __restrict__ Pin, double* __restrict__ Pout,
                                                     double* __restrict__ U0, double* __restrict__ U,
                                                     FluxView V, GridDesc G, PhysParams pp, double b, int stage,
                                                     const double* __restrict__ dtp, DevStatus* __restrict__ st,
                                                     const double* __restrict__ S)
{
    constexpr int NQ = LawInfo<LAW>::NQ;
    if (st->code != 0 || st->halt || st->done) return;
    const int ii = blockIdx.x * blockDim.x + threadIdx.x;
    if (ii >= G.n[0]) return;
    const int jj = blockIdx.y, kk = blockIdx.z;
    const int i = ii + G.g[0], j = jj + G.g[1], k = kk + G.g[2];
    const long long pc = ((long long) k * G.N[1] + j) * G.N[0] + i;
    const long long uc = ((long long) kk * G.n[1] + jj) * G.n[0] + ii;
    const double dt = *dtp;
    const double factor = -1.0;
    const double A1000 = G.dA[0], A0000 = G.dA[0], A0101 = G.dA[1], A0001 = G.dA[1];
    const double A0012 = G.dA[2], A0002 = G.dA[2];
    const double vol = G.dV;
    const bool fx = G.n[0] > 1, fy = G.n[1] > 1, fz = G.n[2] > 1;

    double Pc[NQ], Uo[NQ], Up[NQ], Un[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) Pc[q] = Pin[q * G.sP + pc];

    if (stage == 0) {
        const int e = law_p2u<LAW>(pp, Pc, Uo);
        if (e != ST_OK) { record_status(st, e); return; }
#pragma unroll
        for (int q = 0; q < NQ; ++q) { U0[q * G.sU + uc] = Uo[q]; Up[q] = Uo[q]; }
    } else {
#pragma unroll
        for (int q = 0; q < NQ; ++q) { Uo[q] = U0[q * G.sU + uc]; Up[q] = U[q * G.sU + uc]; }
    }

#pragma unroll
    for (int q = 0; q < NQ; ++q) {
        const double fxp = fx ? face_flux<NQ>(V, G, 0, q, i + 1, j, k) : 0.0;
        const double fxm = fx ? face_flux<NQ>(V, G, 0, q, i, j, k) : 0.0;
        const double fyp = fy ? face_flux<NQ>(V, G, 1, q, i, j + 1, k) : 0.0;
        const double fym = fy ? face_flux<NQ>(V, G, 1, q, i, j, k) : 0.0;
        const double fzp = fz ? face_flux<NQ>(V, G, 2, q, i, j, k + 1) : 0.0;
        const double fzm = fz ? face_flux<NQ>(V, G, 2, q, i, j, k) : 0.0;
        double L = factor / vol * (+fxp * A1000 - fxm * A0000 + fyp * A0101 - fym * A0001
                                   + fzp * A0012 - fzm * A0002);
        if constexpr (LAW == LAW_MHD_COOL) {
            // NewtonianMHD::addSourceTerms (ConservationLaws.cpp:489-501)
            if (q == 4) L -= Pc[4] / (pp.gamma - 1.0) * pp.cooling_rate;
            if (q == 8) L += Pc[4] / (pp.gamma - 1.0) * pp.cooling_rate;
        }
        if (S) L += S[q * G.sP + pc];  // the source terms function's array (SolutionSchemes.cpp:219-228)
        Un[q] = Uo[q] * (1 - b) + (Up[q] + dt * L) * b;
        U[q * G.sU + uc] = Un[q];
    }

    double Pn[NQ];
    int code = ST_OK;
    const int e = law_cons<LAW>(pp, Un, Pn, &code);
    if (e == ST_INVERSION_FAILURE) {
        atomicAdd(&st->failures, 1);
        const unsigned long long z = (unsigned long long) uc;
        const unsigned long long prev = atomicMin(&st->first_zone, z);
        if (z < prev) atomicExch(&st->first_code, code);
#pragma unroll
        for (int q = 0; q < NQ; ++q) Pn[q] = Pc[q]; // a failed zone keeps its value
    } else if (e != ST_OK) {
        record_status(st, e);
        return;
    }

    // the zone's cell, then (zones within a guard width of an edge) its guard
    // images on every combination of axes
    for (int c = 0; c <= G.g[2]; ++c) {
        int oz, sz;
        if (!guard_image(c, kk, G.n[2], G.g[2], G.bc, oz, sz)) continue;
        for (int bb = 0; bb <= G.g[1]; ++bb) {
            int oy, sy;
            if (!guard_image(bb, jj, G.n[1], G.g[1], G.bc, oy, sy)) continue;
            for (int a = 0; a <= G.g[0]; ++a) {
                int ox, sx;
                if (!guard_image(a, ii, G.n[0], G.g[0], G.bc, ox, sx)) continue;
                const long long o = ((long long) oz * G.N[1] + oy) * G.N[0] + ox;
#pragma unroll
                for (int q = 0; q < NQ; ++q) {
                    double v = Pn[q];
                    if ((q == 1 && sx) || (q == 2 && sy) || (q == 3 && sz)) v *= -1;
                    Pout[q * G.sP + o] = v;
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------
// FieldOperator::getCourantTimestep: min over interior zones of
// lmin / max_direction(maxEigenvalueMagnitude).  Positive doubles order like
// their bit patterns, so the minimum is an atomicMin on the bits; NaN and
// +inf (bit patterns above DBL_MAX) never win, as in the reference's
// "if (dt < courantTimestep)" starting from DBL_MAX.
template <int LAW>
__global__ void __launch_bounds__(256) courant_kernel(const double* __restrict__ P, GridDesc G, PhysParams pp,
                                                      DevStatus* __restrict__ st)
{
    constexpr int NQ = LawInfo<LAW>::NQ;
    const int ii = blockIdx.x * blockDim.x + threadIdx.x;
    const int jj = blockIdx.y, kk = blockIdx.z;
    unsigned long long mine = ~0ull;
    if (ii < G.n[0] && st->code == 0) {
        const long long pc = ((long long) (kk + G.g[2]) * G.N[1] + (jj + G.g[1])) * G.N[0] + (ii + G.g[0]);
        double Pc[NQ];
#pragma unroll
        for (int q = 0; q < NQ; ++q) Pc[q] = P[q * G.sP + pc];
        double lam[3];
        int e = ST_OK;
        for (int a = 0; a < 3 && e == ST_OK; ++a) {
            StateD<NQ> S;
            e = law_prim<LAW>(pp, Pc, G.nrm[a], S);
            lam[a] = max_eigen_magnitude<NQ>(S.A);
        }
        if (e != ST_OK) {
            record_status(st, e);
        } else {
            double lmax = lam[0];
            if (lmax < lam[1]) lmax = lam[1];
            if (lmax < lam[2]) lmax = lam[2];
            const double dt = G.lmin / lmax;
            if (dt < 1.7976931348623157e308) mine = (unsigned long long) __double_as_longlong(dt);
        }
    }
    // warp then block minimum
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const unsigned long long o = __shfl_down_sync(0xffffffffu, mine, off);
        mine = o < mine ? o : mine;
    }
    __shared__ unsigned long long red[8];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) red[w] = mine;
    __syncthreads();
    if (w == 0) {
        mine = lane < (blockDim.x >> 5) ? red[lane] : ~0ull;
#pragma unroll
        for (int off = 4; off > 0; off >>= 1) {
            const unsigned long long o = __shfl_down_sync(0xffffffffu, mine, off);
            mine = o < mine ? o : mine;
        }
        if (lane == 0 && mine != ~0ull) atomicMin(&st->dt_bits, mine);
    }
}

// ---------------------------------------------------------------------------
static PhysParams to_dev(const PhysParamsH& h)
{
    PhysParams p;
    p.gamma = h.gamma;
    p.plm_theta = h.plm_theta;
    p.shenzha_A = h.shenzha_A;
    p.pressure_floor = h.pressure_floor;
    p.weno_is = h.weno_is;
    p.cooling_rate = h.cooling_rate;
    return p;
}

template <int LAW, int RECON, int RIEMANN>
static void flux_launch(int axis, const GridDesc& G, const PhysParams& pp, const double* P, double* F,
                        DevStatus* st, cudaStream_t s)
{
    // faces along the axis: the interior faces; across: interior rows, plus
    // one guard row per side on fleshed axes when flux CT is on
    int lo[3], nb[3];
    for (int a = 0; a < 3; ++a) {
        if (a == axis) { lo[a] = G.g[a]; nb[a] = G.n[a] + 1; }
        else if (G.n[a] > 1) { const int e = G.ct ? 1 : 0; lo[a] = G.g[a] - e; nb[a] = G.n[a] + 2 * e; }
        else { lo[a] = 0; nb[a] = 1; }
    }
    dim3 block(128), grid((unsigned) (((long long) nb[0] * nb[1] + 127) / 128), nb[2]);
    flux_kernel<LAW, RECON, RIEMANN><<<grid, block, 0, s>>>(P, F, G, pp, axis, lo[0], lo[1], lo[2], nb[0], nb[1], st);
}

template <int LAW, int RECON>
static void flux_dispatch_r(int riemann, int axis, const GridDesc& G, const PhysParams& pp, const double* P,
                            double* F, DevStatus* st, cudaStream_t s)
{
    if (riemann == RIEMANN_HLLC) flux_launch<LAW, RECON, RIEMANN_HLLC>(axis, G, pp, P, F, st, s);
    else flux_launch<LAW, RECON, RIEMANN_HLLE>(axis, G, pp, P, F, st, s);
}

template <int LAW>
static void flux_dispatch(int recon, int riemann, int axis, const GridDesc& G, const PhysParams& pp,
                          const double* P, double* F, DevStatus* st, cudaStream_t s)
{
    switch (recon) {
        case RECON_PCM: flux_dispatch_r<LAW, RECON_PCM>(riemann, axis, G, pp, P, F, st, s); break;
        case RECON_PLM: flux_dispatch_r<LAW, RECON_PLM>(riemann, axis, G, pp, P, F, st, s); break;
        default: flux_dispatch_r<LAW, RECON_WENO5>(riemann, axis, G, pp, P, F, st, s); break;
    }
}

void plain_flux(int law, int recon, int riemann, int axis, const GridDesc& G, const PhysParamsH& ph,
                const double* P, double* F, DevStatus* st, cudaStream_t s)
{
    const PhysParams pp = to_dev(ph);
    switch (law) {
        case LAW_HYDRO: flux_dispatch<LAW_HYDRO>(recon, riemann, axis, G, pp, P, F, st, s); break;
        case LAW_MHD: flux_dispatch<LAW_MHD>(recon, riemann, axis, G, pp, P, F, st, s); break;
        case LAW_MHD_COOL: flux_dispatch<LAW_MHD_COOL>(recon, riemann, axis, G, pp, P, F, st, s); break;
        default: flux_dispatch<LAW_RMHD>(recon, riemann, axis, G, pp, P, F, st, s); break;
    }
}

void plain_update(int law, const GridDesc& G, const PhysParamsH& ph, const double* Pin, double* Pout,
                  double* U0, double* U, const double* Fx, const double* Fy, const double* Fz,
                  double b, int stage, const double* dt, DevStatus* st, cudaStream_t s, const double* S)
{
    const PhysParams pp = to_dev(ph);
    FluxView V;
    V.F[0] = Fx; V.F[1] = Fy; V.F[2] = Fz;
    V.sF = G.sF;
    V.M0 = G.N[0] + 1;
    V.M1 = G.N[1] + 1;
    dim3 block(128), grid((G.n[0] + 127) / 128, G.n[1], G.n[2]);
    switch (law) {
        case LAW_HYDRO: update_kernel<LAW_HYDRO><<<grid, block, 0, s>>>(Pin, Pout, U0, U, V, G, pp, b, stage, dt, st, S); break;
        case LAW_MHD: update_kernel<LAW_MHD><<<grid, block, 0, s>>>(Pin, Pout, U0, U, V, G, pp, b, stage, dt, st, S); break;
        case LAW_MHD_COOL: update_kernel<LAW_MHD_COOL><<<grid, block, 0, s>>>(Pin, Pout, U0, U, V, G, pp, b, stage, dt, st, S); break;
        default: update_kernel<LAW_RMHD><<<grid, block, 0, s>>>(Pin, Pout, U0, U, V, G, pp, b, stage, dt, st, S); break;
    }
}

void plain_courant(int law, const GridDesc& G, const PhysParamsH& ph, const double* P, DevStatus* st,
                   cudaStream_t s)
{
    const PhysParams pp = to_dev(ph);
    dim3 block(256), grid((G.n[0] + 255) / 256, G.n[1], G.n[2]);
    switch (law) {
        case LAW_HYDRO: courant_kernel<LAW_HYDRO><<<grid, block, 0, s>>>(P, G, pp, st); break;
        case LAW_MHD: courant_kernel<LAW_MHD><<<grid, block, 0, s>>>(P, G, pp, st); break;
        case LAW_MHD_COOL: courant_kernel<LAW_MHD_COOL><<<grid, block, 0, s>>>(P, G, pp, st); break;
        default: courant_kernel<LAW_RMHD><<<grid, block, 0, s>>>(P, G, pp, st); break;
    }
}

} // namespace mara

// ---------------------------------------------------------------------------
// The ready-made uniform-gravity source terms function (include/mara_gpu.h).
__global__ void k_uniform_gravity(const double* __restrict__ P, double* __restrict__ S, long long sP, long long cells,
                                  int nq, double g1, double g2, double g3)
{
    const long long c = blockIdx.x * (long long) blockDim.x + threadIdx.x;
    if (c >= cells) return;
    const double rho = P[c], v1 = P[sP + c], v2 = P[2 * sP + c], v3 = P[3 * sP + c];
    S[c] = 0.0;
    S[sP + c] = rho * g1;
    S[2 * sP + c] = rho * g2;
    S[3 * sP + c] = rho * g3;
    S[4 * sP + c] = rho * (v1 * g1 + v2 * g2 + v3 * g3);
    for (int q = 5; q < nq; ++q) S[q * sP + c] = 0.0;
}

extern "C" int mara_source_uniform_gravity(void* user, const MaraSourceTermsArgs* a)
{
    if (!user || !a) return MARA_ERR_ARGUMENT;
    const double* g = (const double*) user;
    const long long cells = (long long) a->N[0] * a->N[1] * a->N[2];
    k_uniform_gravity<<<(unsigned) ((cells + 255) / 256), 256, 0, (cudaStream_t) a->stream>>>(
        a->P, a->S, a->sP, cells, a->nq, g[0], g[1], g[2]);
    return cudaGetLastError() == cudaSuccess ? MARA_OK : MARA_ERR_CUDA;
}
