// hydro_cluster.cuh -- many driver-loop steps of a small 1-D hydro grid in one
// launch, on one thread-block cluster (mixed precision, the arithmetic of
// the fused stage kernel in hydro_tile.cuh).
//
// A 1-D grid of up to CLUSTER1D_MAX_CTAS x 1024 zones stays in the shared
// memory of a cluster of C CTAs for the whole launch: CTA r holds zones
// [r m, (r + 1) m) of the FP32-pair state and of U0.  Per RK stage each CTA
// converts its zones to primitives, the cluster synchronises, each CTA reads
// its stencil-wide halo from its neighbours' shared memory (distributed
// shared memory) or from the boundary image of the grid's edge, computes its
// faces and updates its zones in place.  The Courant step of the new state is
// reduced across the cluster through shared memory too, so the next step's
// dt = min(cfl x courant, t_final - t) (src/Problems.cpp:181-186) is known to
// every CTA without leaving the SMs.  Per step this replaces three kernel
// launches and the passes over the state in HBM with two cluster barriers
// per stage: a small grid is latency-bound, not bandwidth-bound.
#pragma once

#include <cooperative_groups.h>
#include <cfloat>

#include "hydro_tile.cuh"
#include "internal.h"

namespace mara {

constexpr int CLUSTER1D_MAX_CTAS = 8;  // portable cluster size
constexpr int CLUSTER1D_WIDE_CTAS = 16; // the non-portable size, where the GPU can place it
constexpr int CLUSTER1D_MAX_ZONES_PER_CTA = 1024;

// dynamic shared memory of a CTA holding m zones with a halo of G: U hi/lo
// and U0 hi/lo (5 fields each), two buffers of primitives with halo (stages
// alternate), face fluxes, two Courant slots (steps alternate)
__host__ __device__ constexpr size_t cluster1d_smem_bytes(int m, int G)
{
    return sizeof(float) * (4 * 5 * (size_t) m + 2 * 5 * (size_t) (m + 2 * G) + 5 * (size_t) (m + 1) + 4);
}

// What one launch advances: cluster c of the launch runs the driver loop of
// slot slots[c] (slot 0 when slots is null) of the tables below, at most
// nsteps steps, stopping at t_final (t_final < 0: no end time).  The tables
// are the handle's status (one slot) or the batch's per-grid arrays.
struct Cluster1DJob {
    const HGrid* grids;          // grid records (device)
    const int* slots;            // slot of each cluster, or null
    double* t;                   // clock, per slot
    long long* steps;
    double* dt;
    int* done;                   // done_value once t reached t_final
    unsigned long long* used;    // the Courant step the last dt came from (may be null)
    unsigned long long* cfl;     // Courant step of the state (bits of a positive double)
    const double* tfin;          // per-slot end times, or null: t_final below
    const double* cflp;          // per-slot CFL numbers, or null: cfl_number below
    double t_final, cfl_number;
    int done_value;
    int order;                   // RK order
    int nsteps;
    int buffer;                  // the state's buffer in the grid's rotation
};

// Driver-loop steps of small 1-D grids; the state is read from and written
// back to buffer job.buffer of each grid's rotation.  Clusters of one launch
// may hold grids of different sizes: each CTA uses the zones of its own grid
// (at most the m the launch's shared memory was sized for).
template <int RECON, int RIEMANN, bool ACC64 = false>
__global__ void __launch_bounds__(1024) hydro_cluster1d_kernel(Cluster1DJob job)
{
    namespace cg = cooperative_groups;
    constexpr int G = HaloOf<RECON>::G;
    cg::cluster_group cluster = cg::this_cluster();
    const int C = (int) cluster.num_blocks();
    const int r = (int) cluster.block_rank();
    const int slot = job.slots ? job.slots[blockIdx.x / C] : 0;
    const HGrid& g = job.grids[slot];
    const int s = job.buffer;
    const int order = job.order;
    const double cfl = job.cflp ? job.cflp[slot] : job.cfl_number;
    const double t_final = job.tfin ? job.tfin[slot] : job.t_final;
    const int n = g.n0;
    const int m = (n + C - 1) / C;                 // zones per CTA
    const int z0 = r * m;
    const int mine = max(0, min(m, n - z0));       // zones this CTA owns

    // the state: FP32 pairs (hi, lo), or with ACC64 the FP64 accumulator's
    // high and low 32-bit halves in the same two arrays
    extern __shared__ float smem[];
    float* Uh = smem;                              // [5][m]
    float* Ul = Uh + 5 * m;
    float* U0h = Ul + 5 * m;
    float* U0l = U0h + 5 * m;
    const int W = m + 2 * G;
    float* Pbuf = U0l + 5 * m;                     // 2 x [5][W], zone z at z + G
    float* Fx = Pbuf + 2 * 5 * W;                  // [5][m + 1]
    float* red = Fx + 5 * (m + 1);                 // this CTA's Courant slots, [2]
    __shared__ float wmin[32];
    float* __restrict__ gh = s == 0 ? g.Uh[0] : s == 1 ? g.Uh[1] : g.Uh[2];
    float* __restrict__ gl = s == 0 ? g.Ul[0] : s == 1 ? g.Ul[1] : g.Ul[2];

    auto acc = [](const float* h, const float* l, int k) {
        return __hiloint2double(__float_as_int(h[k]), __float_as_int(l[k]));
    };
    auto set_acc = [](float* h, float* l, int k, double v) {
        h[k] = __int_as_float(__double2hiint(v));
        l[k] = __int_as_float(__double2loint(v));
    };
    for (int i = threadIdx.x; i < mine; i += blockDim.x) {
#pragma unroll
        for (int q = 0; q < 5; ++q) {
            if constexpr (ACC64) {
                set_acc(Uh, Ul, q * m + i, reinterpret_cast<const double*>(gh)[q * g.sU + z0 + i]);
            } else {
                Uh[q * m + i] = gh[q * g.sU + z0 + i];
                Ul[q * m + i] = gl[q * g.sU + z0 + i];
            }
        }
    }
    // every CTA follows the same clock: the same doubles from the same inputs
    double t = job.t[slot];
    long long steps = job.steps[slot];
    int done = job.done[slot] == job.done_value;
    double dt = job.dt[slot];
    unsigned long long bits = job.cfl[slot];
    unsigned long long used = job.used ? job.used[slot] : 0ull;

    // One cluster barrier per RK stage, after the primitives are formed: the
    // primitives alternate between two buffers by stage, so a neighbour's
    // halo reads of one stage end (it reaches the next barrier) before this
    // CTA writes that buffer again two stages later; the Courant slots
    // alternate by step, read by every CTA after the first barrier of the
    // next step and written again after the second.
    int par = 0;                                   // the stage's buffer
    int step = 0;
    for (; step < job.nsteps && !done; ++step) {
        float zdt = 3.0e38f;
        for (int rk = 0; rk < order; ++rk, par ^= 1) {
            const int last = rk == order - 1;
            const float b = order == 1 ? 1.f : order == 2 ? (rk == 0 ? 1.f : 0.5f)
                                                          : (rk == 0 ? 1.f : rk == 1 ? 0.25f : 2.f / 3.f);
            const float omb = 1.f - b;
            float* Ps = Pbuf + par * 5 * W;
            // 1. primitives of the owned zones (from the high words, or the
            //    accumulator rounded to FP32)
            for (int i = threadIdx.x; i < mine; i += blockDim.x) {
                float U[5], P[5];
#pragma unroll
                for (int q = 0; q < 5; ++q) U[q] = ACC64 ? d2f_rn_ftz(acc(Uh, Ul, q * m + i)) : Uh[q * m + i];
                fh_cons(g.gamma, U, P);
#pragma unroll
                for (int q = 0; q < 5; ++q) Ps[q * W + G + i] = P[q];
            }
            cluster.sync();
            if (rk == 0) {
                // the step start of the fused path (k_fused_run_begin): the
                // Courant step of the state, from the previous step's slots
                // (the first step of a launch takes the one it was given)
                if (step > 0) {
                    float mn = 3.0e38f;
                    for (int k = 0; k < C; ++k) mn = fminf(mn, cluster.map_shared_rank(red, k)[(step - 1) & 1]);
                    // no valid zone leaves the slot at its reset value, as in the fused path
                    bits = (unsigned long long) __double_as_longlong(mn < 3.0e38f ? (double) mn : DBL_MAX);
                }
                used = bits;
                dt = cfl * __longlong_as_double((long long) bits);
                if (t_final >= 0.0) {
                    if (!(t < t_final)) { done = 1; break; }
                    const double dt2 = t_final - t;
                    dt = dt < dt2 ? dt : dt2;
                }
            }
            const float dtf = (float) dt;
            // 2. the halo: 2G zones from the neighbours' shared memory, or the
            //    boundary image of the grid's edge (momentum negated across a
            //    reflecting boundary)
            if (threadIdx.x < 2 * G) {
                const int k = threadIdx.x;
                const int local = k < G ? k - G : mine + (k - G);  // zone index relative to z0
                int flip = 0;
                const int z = bc_image(z0 + local, n, g.bc, flip);
                const int owner = z / m, at = z - owner * m;
                const float* src = cluster.map_shared_rank(Ps, owner);
#pragma unroll
                for (int q = 0; q < 5; ++q) {
                    float v = src[q * W + G + at];
                    if (flip && q == 1) v = -v;
                    Ps[q * W + G + local] = v;
                }
            }
            __syncthreads();
            // 3. faces: face f sits left of owned zone f, f = 0..mine
            for (int f = threadIdx.x; f <= mine; f += blockDim.x) {
                float PL[5], PR[5], Fh[5];
#pragma unroll
                for (int q = 0; q < 5; ++q) {
                    float v[2 * G];
#pragma unroll
                    for (int c = 0; c < 2 * G; ++c) v[c] = Ps[q * W + f + c];
                    recon_pair<RECON>(v, g.plm_theta, PL[q], PR[q]);
                }
                hydro_face_flux<RIEMANN, 0>(g.gamma, PL, PR, Fh);
#pragma unroll
                for (int q = 0; q < 5; ++q) Fx[q * (m + 1) + f] = Fh[q];
            }
            __syncthreads();
            // 4. divergence and RK combine, in place; U0 is the step's start
            for (int i = threadIdx.x; i < mine; i += blockDim.x) {
                float Unew[5];
#pragma unroll
                for (int q = 0; q < 5; ++q) {
                    const float L = fh_div(Fx[q * (m + 1) + i], Fx[q * (m + 1) + i + 1], g.idx);
                    if constexpr (ACC64) {
                        // rk_combine_d as the tile kernels' FP64-accumulator update
                        const double Upd = acc(Uh, Ul, q * m + i);
                        if (rk == 0) set_acc(U0h, U0l, q * m + i, Upd);
                        const double Un = rk_combine_d(rk == 0 ? 0.0 : acc(U0h, U0l, q * m + i), Upd, f_mul(dtf, L), b);
                        set_acc(Uh, Ul, q * m + i, Un);
                        Unew[q] = d2f_rn_ftz(Un);
                        continue;
                    }
                    const df Up = {Uh[q * m + i], Ul[q * m + i]};
                    df U0 = Up;
                    if (rk == 0) {
                        U0h[q * m + i] = Up.hi;
                        U0l[q * m + i] = Up.lo;
                    } else {
                        U0 = {U0h[q * m + i], U0l[q * m + i]};
                    }
                    const df Un = rk_combine(U0, Up, f_mul(dtf, L), b, omb);
                    Uh[q * m + i] = Un.hi;
                    Ul[q * m + i] = Un.lo;
                    Unew[q] = Un.hi;
                }
                if (last) zdt = fminf(zdt, hydro_zone_dt(g, Unew));
            }
            if (last) {
                // this CTA's part of the new state's Courant step: the minimum
                // of the valid zone steps, as block_min_to orders them
                float v = (zdt > 0.f && zdt < 3.0e38f) ? zdt : 3.0e38f;
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) v = fminf(v, __shfl_down_sync(0xffffffffu, v, off));
                if ((threadIdx.x & 31) == 0) wmin[threadIdx.x >> 5] = v;
                __syncthreads();
                if (threadIdx.x == 0) {
                    float w = 3.0e38f;
                    for (int k = 0; k < (int) (blockDim.x + 31) / 32; ++k) w = fminf(w, wmin[k]);
                    red[step & 1] = w;
                }
            }
        }
        if (done) break;
        t += dt;
        steps += 1;
        // the next step's start would stop here: stop now, so that a grid
        // finishing on a launch's last step is reported by that launch
        if (t_final >= 0.0 && !(t < t_final)) { done = 1; ++step; break; }
    }
    // the Courant step of the last step taken, once every CTA's slot is in
    cluster.sync();
    if (step > 0) {
        float mn = 3.0e38f;
        for (int k = 0; k < C; ++k) mn = fminf(mn, cluster.map_shared_rank(red, k)[(step - 1) & 1]);
        bits = (unsigned long long) __double_as_longlong(mn < 3.0e38f ? (double) mn : DBL_MAX);
    }
    for (int i = threadIdx.x; i < mine; i += blockDim.x) {
#pragma unroll
        for (int q = 0; q < 5; ++q) {
            if constexpr (ACC64) {
                // the accumulator and its FP32 copy (read by the tile kernels' halo staging)
                const double v = acc(Uh, Ul, q * m + i);
                reinterpret_cast<double*>(gh)[q * g.sU + z0 + i] = v;
                gl[q * g.sU + z0 + i] = d2f_rn_ftz(v);
            } else {
                gh[q * g.sU + z0 + i] = Uh[q * m + i];
                gl[q * g.sU + z0 + i] = Ul[q * m + i];
            }
        }
    }
    // the clock is published after every CTA's part of the state; the slots
    // are read before any CTA leaves
    __threadfence();
    cluster.sync();
    if (r == 0 && threadIdx.x == 0) {
        job.t[slot] = t;
        job.steps[slot] = steps;
        job.dt[slot] = dt;
        if (job.used) job.used[slot] = used;
        job.cfl[slot] = bits;
        __threadfence();
        if (done) job.done[slot] = job.done_value;
    }
}

// grid of cluster_count clusters of C CTAs, each CTA sized for up to m zones
// the launch configuration of cluster_count clusters of C CTAs sized for up
// to m zones each (at[] must outlive the returned configuration)
template <int RECON, int RIEMANN, bool ACC64 = false>
inline cudaError_t cluster1d_config(int cluster_count, int C, int m, cudaStream_t stream, cudaLaunchAttribute* at,
                                    cudaLaunchConfig_t& lc)
{
    constexpr int G = HaloOf<RECON>::G;
    const size_t smem = cluster1d_smem_bytes(m, G);
    const int threads = m + 1 < 1024 ? ((m + 1 + 31) / 32) * 32 : 1024;  // one thread per face
    auto k = hydro_cluster1d_kernel<RECON, RIEMANN, ACC64>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
    if (e == cudaSuccess && C > CLUSTER1D_MAX_CTAS)
        e = cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return e;
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned) C;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    lc = {};
    lc.gridDim = dim3((unsigned) (cluster_count * C));
    lc.blockDim = dim3((unsigned) threads);
    lc.dynamicSmemBytes = smem;
    lc.stream = stream;
    lc.attrs = at;
    lc.numAttrs = 1;
    return cudaSuccess;
}

// grid of cluster_count clusters of C CTAs, each CTA sized for up to m zones
template <int RECON, int RIEMANN, bool ACC64 = false>
inline cudaError_t launch_cluster1d(const Cluster1DJob& job, int cluster_count, int C, int m, cudaStream_t stream)
{
    cudaLaunchAttribute at[1];
    cudaLaunchConfig_t lc;
    const cudaError_t e = cluster1d_config<RECON, RIEMANN, ACC64>(cluster_count, C, m, stream, at, lc);
    if (e != cudaSuccess) return e;
    return cudaLaunchKernelEx(&lc, hydro_cluster1d_kernel<RECON, RIEMANN, ACC64>, job);
}

// can the GPU place one cluster of C CTAs sized for m zones?
template <int RECON, int RIEMANN, bool ACC64 = false>
inline bool cluster1d_fits(int C, int m)
{
    cudaLaunchAttribute at[1];
    cudaLaunchConfig_t lc;
    int n = 0;
    if (cluster1d_config<RECON, RIEMANN, ACC64>(1, C, m, nullptr, at, lc) != cudaSuccess ||
        cudaOccupancyMaxActiveClusters(&n, hydro_cluster1d_kernel<RECON, RIEMANN, ACC64>, &lc) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return n > 0;
}

// CTAs of a grid of n zones: every CTA owns at least 128 zones, at most
// `cap` CTAs
inline int cluster1d_ctas(int n, int cap = CLUSTER1D_MAX_CTAS)
{
    const int c = n / 128;
    return c < 1 ? 1 : c > cap ? cap : c;
}

} // namespace mara
