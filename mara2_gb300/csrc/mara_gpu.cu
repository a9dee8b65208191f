// mara_gpu.cu -- the C ABI (include/mara_gpu.h): handle life cycle, layout
// transposes between the reference's AoS MeshData::P and the device SoA
// state, the RK stage sequence of MethodOfLinesTVD::advance, the device-side
// driver loop and its CUDA graphs.
#include <cuda_runtime.h>

#include <cfloat>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/mara_gpu.h"
#include "diagnostics.cuh"
#include "internal.h"
#include "mixed.h"

using namespace mara;

namespace mara {

// ---------------------------------------------------------------------------
// small device helpers
__global__ void k_courant_init(DevStatus* st)
{
    const double big = DBL_MAX;
    st->dt_bits = (unsigned long long) __double_as_longlong(big);
}

// dt = min(cfl * courant, t_final - t) as the regression drivers compute it
// (src/Problems.cpp:181-186); a step at t >= t_final is not taken.
__global__ void k_dt_from_courant(DevStatus* st, double cfl, double t_final)
{
    if (st->done) return;
    const double courant = __longlong_as_double((long long) st->dt_bits);
    double dt = cfl * courant;
    if (t_final >= 0.0) {
        if (!(st->t < t_final)) { st->done = 1; return; }
        const double dt2 = t_final - st->t;
        dt = dt < dt2 ? dt : dt2;
    }
    st->dt = dt;
}

// an advance with a given dt is always taken (SolutionScheme::advance), also
// after a driver loop stopped at t_final
__global__ void k_set_dt(DevStatus* st, double dt)
{
    st->dt = dt;
    st->done = 0;
}

// an advance that ran counts toward the state's ping-pong parity
__global__ void k_step_taken(DevStatus* st)
{
    if (!st->done && !st->code && !st->halt) st->taken += 1;
}

__global__ void k_advance_time(DevStatus* st)
{
    if (st->done || st->code) return;
    st->t += st->dt;
    st->steps += 1;
    st->taken += 1;
}

__global__ void k_status_reset(DevStatus* st)
{
    DevStatus z;
    memset(&z, 0, sizeof(z));
    z.first_zone = ~0ull;
    *st = z;
}

__global__ void k_run_begin(DevStatus* st, double t)
{
    st->t = t;
    st->steps = 0;
    st->done = 0;
}

// AoS (i, j, k, q), q fastest  <->  SoA q * sP + (k * N1 + j) * N0 + i, over
// the AoS cells [c0, c1)
// AoS (k fastest, the reference's MeshData::P) <-> SoA (x fastest).  A
// block's cells are one contiguous slab of the AoS array, moved with
// consecutive threads on consecutive doubles (the array may be the caller's
// page-locked host memory, reached over the chip-to-chip link) and
// transposed in shared memory.
constexpr int CONV_BLOCK = 256;
constexpr int CONV_MAXQ = 10;  // MARA_NUM_FIELDS: the most fields any law carries (NewtonianMHD with cooling: 9)

__device__ __forceinline__ long long soa_index(long long c, const GridDesc& G)
{
    const int k = (int) (c % G.N[2]);
    const int j = (int) ((c / G.N[2]) % G.N[1]);
    const int i = (int) (c / ((long long) G.N[2] * G.N[1]));
    return ((long long) k * G.N[1] + j) * G.N[0] + i;
}

__global__ void __launch_bounds__(CONV_BLOCK) k_aos_to_soa(const double* __restrict__ aos, double* __restrict__ soa,
                                                           GridDesc G, long long c0, long long c1)
{
    __shared__ double slab[CONV_BLOCK * CONV_MAXQ];
    const int nq = G.nq;
    const long long b0 = c0 + blockIdx.x * (long long) CONV_BLOCK;
    const int nc = (int) min((long long) CONV_BLOCK, c1 - b0);
    for (int e = threadIdx.x; e < nc * nq; e += CONV_BLOCK) slab[e] = aos[b0 * nq + e];
    __syncthreads();
    if (threadIdx.x >= nc) return;
    const long long s = soa_index(b0 + threadIdx.x, G);
    for (int q = 0; q < nq; ++q) soa[q * G.sP + s] = slab[threadIdx.x * nq + q];
}

__global__ void __launch_bounds__(CONV_BLOCK) k_soa_to_aos(const double* __restrict__ soa, double* __restrict__ aos,
                                                           GridDesc G, long long c0, long long c1)
{
    __shared__ double slab[CONV_BLOCK * CONV_MAXQ];
    const int nq = G.nq;
    const long long b0 = c0 + blockIdx.x * (long long) CONV_BLOCK;
    const int nc = (int) min((long long) CONV_BLOCK, c1 - b0);
    if (threadIdx.x < nc) {
        const long long s = soa_index(b0 + threadIdx.x, G);
        for (int q = 0; q < nq; ++q) slab[threadIdx.x * nq + q] = soa[q * G.sP + s];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < nc * nq; e += CONV_BLOCK) aos[b0 * nq + e] = slab[e];
}

// ---- initial data on the device ----------------------------------------------
// interior coordinate of full index i along an axis (n interior, g guards),
// as the boundary condition's guard fill maps it; flip marks a reflection
__device__ __forceinline__ int bc_interior(int i, int n, int g, int bc, int& flip)
{
    const int x = i - g;
    if (g == 0 || (x >= 0 && x < n)) return x;
    if (bc == BC_PERIODIC) return x < 0 ? x + n : x - n;
    if (bc == BC_OUTFLOW) return x < 0 ? 0 : n - 1;
    flip = 1;
    return x < 0 ? -1 - x : 2 * n - 1 - x;
}

struct GenGeom {
    double lower[3], dx[3];
};

__global__ void k_generate(double* __restrict__ aos, GridDesc G, GenGeom geo, MaraInitialData d)
{
    const long long total = (long long) G.N[0] * G.N[1] * G.N[2];
    const long long c = blockIdx.x * (long long) blockDim.x + threadIdx.x;  // AoS order, k fastest
    if (c >= total) return;
    const int k = (int) (c % G.N[2]);
    const int j = (int) ((c / G.N[2]) % G.N[1]);
    const int i = (int) (c / ((long long) G.N[2] * G.N[1]));
    int f[3] = {0, 0, 0};
    const int ii = bc_interior(i, G.n[0], G.g[0], G.bc, f[0]);
    const int jj = bc_interior(j, G.n[1], G.g[1], G.bc, f[1]);
    const int kk = bc_interior(k, G.n[2], G.g[2], G.bc, f[2]);
    const double x = geo.lower[0] + geo.dx[0] * ((double) ii + 0.5);
    const double y = geo.lower[1] + geo.dx[1] * ((double) jj + 0.5);
    const double z = geo.lower[2] + geo.dx[2] * ((double) kk + 0.5);
    bool left;
    if (d.kind == MARA_INIT_PLANAR_RIEMANN) {
        left = (x - d.x0[0]) * d.normal[0] + (y - d.x0[1]) * d.normal[1] + (z - d.x0[2]) * d.normal[2] < 0;
    } else if (d.kind == MARA_INIT_SHEAR_LAYER) {
        left = fabs(y - d.x0[1]) < d.radius;
    } else {
        const double rx = x - d.x0[0], ry = y - d.x0[1];
        left = sqrt(rx * rx + ry * ry) < d.radius;
    }
    double P[8];
    for (int q = 0; q < G.nq; ++q) P[q] = left ? d.left[q] : d.right[q];
    if (d.kind == MARA_INIT_SHEAR_LAYER && d.noise != 0.0) {
        // SplitMix64 (Steele, Lea & Flood 2014), output number m + 1
        const unsigned long long m = ((unsigned long long) ii * G.n[1] + jj) * G.n[2] + kk;
        unsigned long long zz = d.seed + (m + 1) * 0x9E3779B97F4A7C15ull;
        zz = (zz ^ (zz >> 30)) * 0xBF58476D1CE4E5B9ull;
        zz = (zz ^ (zz >> 27)) * 0x94D049BB133111EBull;
        zz ^= zz >> 31;
        const double u = (double) (zz >> 11) * (1.0 / 9007199254740992.0);
        P[2] = (-1.0 + 2.0 * u) * d.noise;
    }
    for (int a = 0; a < 3; ++a)
        if (f[a]) P[1 + a] *= -1;
    for (int q = 0; q < G.nq; ++q) aos[c * G.nq + q] = P[q];
}

// ---- the divergence-free field from a vector potential (Problems.cpp:660-667)
// A(face index n, component, face axis) over the (N + 1)^3 face index space
struct VecPot {
    const double* A;
    int f0, f1, f2;
    // CellCenteredFieldCT::vectorPotentialToFluxes (CellCenteredFieldCT.cpp:
    // 136-150): flux of field component q through faces of axis a
    __device__ __forceinline__ double F(int i, int j, int k, int q, int a) const
    {
        const double* p = A + (((long long) i * f1 + j) * f2 + k) * 9;
        if (a == 0) return q == 1 ? -p[2 * 3 + 0] : q == 2 ? +p[1 * 3 + 0] : 0.0;
        if (a == 1) return q == 2 ? -p[0 * 3 + 1] : q == 0 ? +p[2 * 3 + 1] : 0.0;
        return q == 0 ? -p[1 * 3 + 2] : q == 1 ? +p[0 * 3 + 2] : 0.0;
    }
    // the fluxes after CellCenteredFieldCT::correctGodunovFluxes with magnetic
    // index 0 (CellCenteredFieldCT.cpp:14-134): normal components zero, the
    // tangential ones the edge-EMF average where the reference's loops reach
    __device__ __forceinline__ double G(int i, int j, int k, int q, int a) const
    {
        if (q == a) return 0.0;
        if (a == 0 && q == 1 && f0 >= 3 && i >= 1 && j >= 1 && j < f1 - 1)
            return 0.125 * (+2 * F(i, j, k, 1, 0) + 1 * F(i, j + 1, k, 1, 0) + 1 * F(i, j - 1, k, 1, 0)
                            - 1 * F(i, j + 1, k, 0, 1) - 1 * F(i - 1, j + 1, k, 0, 1)
                            - 1 * F(i, j, k, 0, 1) - 1 * F(i - 1, j, k, 0, 1));
        if (a == 0 && q == 2 && f0 >= 3 && i >= 1 && k >= 1 && k < f2 - 1)
            return 0.125 * (+2 * F(i, j, k, 2, 0) + 1 * F(i, j, k + 1, 2, 0) + 1 * F(i, j, k - 1, 2, 0)
                            - 1 * F(i, j, k + 1, 0, 2) - 1 * F(i - 1, j, k + 1, 0, 2)
                            - 1 * F(i, j, k, 0, 2) - 1 * F(i - 1, j, k, 0, 2));
        if (a == 1 && q == 2 && f1 >= 3 && j >= 1 && k >= 1 && k < f2 - 1)
            return 0.125 * (+2 * F(i, j, k, 2, 1) + 1 * F(i, j, k + 1, 2, 1) + 1 * F(i, j, k - 1, 2, 1)
                            - 1 * F(i, j, k + 1, 1, 2) - 1 * F(i, j - 1, k + 1, 1, 2)
                            - 1 * F(i, j, k, 1, 2) - 1 * F(i, j - 1, k, 1, 2));
        if (a == 1 && q == 0 && f1 >= 3 && i >= 1 && i < f0 - 1 && j >= 1)
            return 0.125 * (+2 * F(i, j, k, 0, 1) + 1 * F(i + 1, j, k, 0, 1) + 1 * F(i - 1, j, k, 0, 1)
                            - 1 * F(i + 1, j, k, 1, 0) - 1 * F(i + 1, j - 1, k, 1, 0)
                            - 1 * F(i, j, k, 1, 0) - 1 * F(i, j - 1, k, 1, 0));
        if (a == 2 && q == 0 && f2 >= 3 && i >= 1 && i < f0 - 1 && k >= 1)
            return 0.125 * (+2 * F(i, j, k, 0, 2) + 1 * F(i + 1, j, k, 0, 2) + 1 * F(i - 1, j, k, 0, 2)
                            - 1 * F(i + 1, j, k, 2, 0) - 1 * F(i + 1, j, k - 1, 2, 0)
                            - 1 * F(i, j, k, 2, 0) - 1 * F(i, j, k - 1, 2, 0));
        if (a == 2 && q == 1 && f2 >= 3 && j >= 1 && j < f1 - 1 && k >= 1)
            return 0.125 * (+2 * F(i, j, k, 1, 2) + 1 * F(i, j + 1, k, 1, 2) + 1 * F(i, j - 1, k, 1, 2)
                            - 1 * F(i, j + 1, k, 2, 1) - 1 * F(i, j + 1, k - 1, 2, 1)
                            - 1 * F(i, j, k, 2, 1) - 1 * F(i, j, k - 1, 2, 1));
        return F(i, j, k, q, a);
    }
};

// Every cell of the AoS staging array (with guards): the magnetic field of
// an interior cell becomes scale x MeshOperator::divergence(G, 1) there
// (MeshOperator.cpp:323-381); a guard cell takes its boundary image's state
// (applySimple: periodic wrap, outflow clamp, reflecting mirror with the
// normal velocity negated), its field computed at the image.  Interior
// threads write only the field components, guard threads read only the
// others, so no thread reads what another writes.
__global__ void k_assign_b(double* __restrict__ aos, GridDesc G, VecPot V, double scale)
{
    const long long total = (long long) G.N[0] * G.N[1] * G.N[2];
    const long long c = blockIdx.x * (long long) blockDim.x + threadIdx.x;  // AoS order, k fastest
    if (c >= total) return;
    const int k = (int) (c % G.N[2]);
    const int j = (int) ((c / G.N[2]) % G.N[1]);
    const int i = (int) (c / ((long long) G.N[2] * G.N[1]));
    int f[3] = {0, 0, 0};
    const int ii = bc_interior(i, G.n[0], G.g[0], G.bc, f[0]) + G.g[0];
    const int jj = bc_interior(j, G.n[1], G.g[1], G.bc, f[1]) + G.g[1];
    const int kk = bc_interior(k, G.n[2], G.g[2], G.bc, f[2]) + G.g[2];
    const double factor = 1.0;
    const double vol = G.dV;
    double* out = aos + c * G.nq;
    for (int q = 0; q < 3; ++q)
        out[5 + q] = factor / vol * (+V.G(ii + 1, jj, kk, q, 0) * G.dA[0] - V.G(ii, jj, kk, q, 0) * G.dA[0]
                                     + V.G(ii, jj + 1, kk, q, 1) * G.dA[1] - V.G(ii, jj, kk, q, 1) * G.dA[1]
                                     + V.G(ii, jj, kk + 1, q, 2) * G.dA[2] - V.G(ii, jj, kk, q, 2) * G.dA[2]) *
                     scale;
    if (ii == i && jj == j && kk == k) return;
    const double* src = aos + (((long long) ii * G.N[1] + jj) * G.N[2] + kk) * G.nq;
    for (int q = 0; q < G.nq; ++q)
        if (q < 5 || q > 7) out[q] = (q >= 1 && q <= 3 && f[q - 1]) ? -src[q] : src[q];
}

void launch_courant_init(DevStatus* st, cudaStream_t s) { k_courant_init<<<1, 1, 0, s>>>(st); }
void launch_dt_from_courant(DevStatus* st, double cfl, double t_final, cudaStream_t s)
{
    k_dt_from_courant<<<1, 1, 0, s>>>(st, cfl, t_final);
}
void launch_set_dt(DevStatus* st, double dt, cudaStream_t s) { k_set_dt<<<1, 1, 0, s>>>(st, dt); }
void launch_advance_time(DevStatus* st, cudaStream_t s) { k_advance_time<<<1, 1, 0, s>>>(st); }
void launch_aos_to_soa_range(const double* aos, double* soa, const GridDesc& G, long long c0, long long c1,
                             cudaStream_t s)
{
    if (c1 <= c0) return;
    k_aos_to_soa<<<(unsigned) ((c1 - c0 + CONV_BLOCK - 1) / CONV_BLOCK), CONV_BLOCK, 0, s>>>(aos, soa, G, c0, c1);
}
void launch_soa_to_aos_range(const double* soa, double* aos, const GridDesc& G, long long c0, long long c1,
                             cudaStream_t s)
{
    if (c1 <= c0) return;
    k_soa_to_aos<<<(unsigned) ((c1 - c0 + CONV_BLOCK - 1) / CONV_BLOCK), CONV_BLOCK, 0, s>>>(soa, aos, G, c0, c1);
}
void launch_aos_to_soa(const double* aos, double* soa, const GridDesc& G, cudaStream_t s)
{
    launch_aos_to_soa_range(aos, soa, G, 0, G.sP, s);
}
void launch_soa_to_aos(const double* soa, double* aos, const GridDesc& G, cudaStream_t s)
{
    launch_soa_to_aos_range(soa, aos, G, 0, G.sP, s);
}

} // namespace mara

// ---------------------------------------------------------------------------
struct TimedPair {
    cudaEvent_t a, b;
    int cls;
};

struct MaraGpuHandle {
    MaraGpuConfig cfg;
    GridDesc G;
    PhysParamsH pp;
    cudaStream_t stream = nullptr;
    cudaStream_t aux = nullptr;          // host <-> device copies, overlapped with conversions
    cudaEvent_t ev[17] = {};             // per-chunk events, [16] joins the streams
    double* P[2] = {nullptr, nullptr};  // primitive state with guards (plain path)
    int cur = 0;                         // P[cur] holds the state once the enqueued steps run
    int cur_base = 0;                    // the parity when the device's count of steps
                                         // taken was last reset
    double* U0 = nullptr;
    double* U = nullptr;
    double* F[3] = {nullptr, nullptr, nullptr};
    double* stage_aos = nullptr;         // device AoS staging for transposes
    DevStatus* st = nullptr;
    DevStatus* st_host = nullptr;        // pinned mirror
    MixedState* mixed = nullptr;         // mixed-precision path
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    double graph_cfl = -1.0, graph_tfinal = -2.0;
    int64_t steps = 0, launches = 0;
    int64_t bytes = 0;
    int timing = 0;
    std::vector<TimedPair> timed;
    double ms_total[3] = {0, 0, 0};
    int64_t timed_launches[3] = {0, 0, 0};
    int last_status = 0;
    MaraGpuStats last_stats;
    double* diag = nullptr;              // diagnostics scratch: partial sums, totals, error word
    MaraSourceTermsFn src_fn = nullptr;  // source terms function (plain path)
    void* src_user = nullptr;
    double* S = nullptr;                 // its output, the layout of P
    int src_error = 0;                   // first non-zero return of src_fn since the last check
};

static int cuda_status(cudaError_t e)
{
    if (e == cudaSuccess) return MARA_OK;
    std::fprintf(stderr, "mara_gpu: CUDA error: %s\n", cudaGetErrorString(e));
    return MARA_ERR_CUDA;
}

#define CK(call) do { const cudaError_t e_ = (call); if (e_ != cudaSuccess) return cuda_status(e_); } while (0)

static int alloc(MaraGpuHandle* h, void** p, size_t bytes)
{
    CK(cudaMalloc(p, bytes));
    CK(cudaMemsetAsync(*p, 0, bytes, h->stream));
    h->bytes += (int64_t) bytes;
    return MARA_OK;
}

// the first non-zero status a source terms function returned since the last call
static int take_source_error(MaraGpuHandle* h)
{
    const int e = h->src_error;
    h->src_error = MARA_OK;
    return e;
}

static void timed_begin(MaraGpuHandle* h, int cls, TimedPair& tp)
{
    tp.cls = cls;
    if (!h->timing) return;
    cudaEventCreate(&tp.a);
    cudaEventCreate(&tp.b);
    cudaEventRecord(tp.a, h->stream);
}

static void timed_end(MaraGpuHandle* h, TimedPair& tp)
{
    if (!h->timing) return;
    cudaEventRecord(tp.b, h->stream);
    h->timed.push_back(tp);
}

static int validate(const MaraGpuConfig* c)
{
    const int n[3] = {c->ni, c->nj, c->nk};
    const int s = c->recon == MARA_RECON_PCM ? 1 : c->recon == MARA_RECON_PLM ? 2 : c->recon == MARA_RECON_WENO5 ? 3 : 0;
    if (c->law < 0 || c->law > 2 || s == 0 || c->riemann < 0 || c->riemann > 1 || c->bc < 0 || c->bc > 2)
        return MARA_ERR_CONFIG;
    if (c->rk_order < 1 || c->rk_order > 3) return MARA_ERR_CONFIG;
    if (c->precision != MARA_PRECISION_FP64 && c->precision != MARA_PRECISION_MIXED &&
        c->precision != MARA_PRECISION_MIXED_FP64)
        return MARA_ERR_CONFIG;
    if (c->law == MARA_LAW_MHD && c->cooling_rate > 0.0 && c->precision != MARA_PRECISION_FP64)
        return MARA_ERR_CONFIG;  // the auxiliary field is on the plain path only
    static_assert(CONV_MAXQ >= 9, "the layout conversions stage up to 9 fields per cell");
    for (int a = 0; a < 3; ++a) {
        if (n[a] < 1 || c->ng[a] < 0) return MARA_ERR_CONFIG;
        if (n[a] == 1 && c->ng[a] != 0) return MARA_ERR_CONFIG;
        if (n[a] > 1 && c->ng[a] < s) return MARA_ERR_GUARD_TOO_SMALL;
        if (n[a] > 1 && n[a] < 2 * c->ng[a]) return MARA_ERR_CONFIG; // guards are images of interior zones
        if (n[a] > 65535 && a > 0) return MARA_ERR_TOO_LARGE;
    }
    if (c->upper[0] <= c->lower[0] || c->upper[1] <= c->lower[1] || c->upper[2] <= c->lower[2])
        return MARA_ERR_CONFIG;
    return MARA_OK;
}

int mara::kernel_law(const MaraGpuConfig* c)
{
    return c->law == MARA_LAW_MHD && c->cooling_rate > 0.0 ? LAW_MHD_COOL : c->law;
}

void mara::make_phys(const MaraGpuConfig* c, PhysParamsH* pp)
{
    pp->gamma = c->gamma;
    pp->plm_theta = c->plm_theta;
    pp->shenzha_A = c->shenzha_A;
    pp->pressure_floor = c->pressure_floor;
    pp->weno_is = c->weno_is;
    pp->cooling_rate = c->cooling_rate;
}

static void make_grid(const MaraGpuConfig* c, GridDesc* G)
{
    const int n[3] = {c->ni, c->nj, c->nk};
    std::memset(G, 0, sizeof(*G));
    double dx[3];
    for (int a = 0; a < 3; ++a) {
        G->n[a] = n[a];
        G->g[a] = c->ng[a];
        G->N[a] = n[a] + 2 * c->ng[a];
        dx[a] = (c->upper[a] - c->lower[a]) / n[a];
    }
    G->nq = c->law == MARA_LAW_HYDRO ? 5 : kernel_law(c) == LAW_MHD_COOL ? 9 : 8;
    G->sP = (long long) G->N[0] * G->N[1] * G->N[2];
    G->sU = (long long) n[0] * n[1] * n[2];
    G->sF = (long long) (G->N[0] + 1) * (G->N[1] + 1) * (G->N[2] + 1);
    G->dA[0] = dx[1] * dx[2];
    G->dA[1] = dx[2] * dx[0];
    G->dA[2] = dx[0] * dx[1];
    G->dV = dx[0] * dx[1] * dx[2];
    G->lmin = dx[0];
    if (dx[1] < G->lmin) G->lmin = dx[1];
    if (dx[2] < G->lmin) G->lmin = dx[2];
    // CartesianMeshGeometry::faceNormal -> UnitVector xhat (0,0), yhat (0,pi/2),
    // zhat (1,0); UnitVector::getCartesianComponents (UnitVector.cpp:32-39).
    // Computed on the host with the same libm calls, so yhat keeps its
    // cos(pi/2) = 6.1e-17 x-component.
    const double mu[3] = {0.0, 0.0, 1.0}, phi[3] = {0.0, M_PI / 2, 0.0};
    for (int a = 0; a < 3; ++a) {
        const double st = std::sqrt(1 - mu[a] * mu[a]);
        G->nrm[a][0] = st * std::cos(phi[a]);
        G->nrm[a][1] = st * std::sin(phi[a]);
        G->nrm[a][2] = mu[a];
    }
    G->bc = c->bc;
    G->ct = (c->law != MARA_LAW_HYDRO) && !c->disable_ct;
}

// The stages of one MethodOfLinesTVD::advance on the plain path; dt is read
// from st->dt on the device.
static void enqueue_plain_step(MaraGpuHandle* h)
{
    static const double b1[1] = {1.0};
    static const double b2[2] = {1.0, 0.5};
    static const double b3[3] = {1.0, 1. / 4, 2. / 3};
    const MaraGpuConfig& c = h->cfg;
    const double* b = c.rk_order == 1 ? b1 : c.rk_order == 2 ? b2 : b3;
    for (int rk = 0; rk < c.rk_order; ++rk) {
        for (int a = 0; a < 3; ++a) {
            if (h->G.n[a] <= 1) continue;
            TimedPair tp;
            timed_begin(h, 0, tp);
            plain_flux(kernel_law(&c), c.recon, c.riemann, a, h->G, h->pp, h->P[h->cur], h->F[a], h->st, h->stream);
            timed_end(h, tp);
            h->launches++;
        }
        const double* S = nullptr;
        if (h->src_fn) {
            MaraSourceTermsArgs a;
            std::memset(&a, 0, sizeof(a));
            a.P = h->P[h->cur];
            a.S = h->S;
            a.sP = h->G.sP;
            a.nq = h->G.nq;
            for (int ax = 0; ax < 3; ++ax) {
                a.N[ax] = h->G.N[ax];
                a.ng[ax] = h->G.g[ax];
                a.lower[ax] = c.lower[ax];
                a.dx[ax] = (c.upper[ax] - c.lower[ax]) / (ax == 0 ? c.ni : ax == 1 ? c.nj : c.nk);
            }
            a.stream = (void*) h->stream;
            const int rc = h->src_fn(h->src_user, &a);
            if (rc != MARA_OK && h->src_error == MARA_OK) h->src_error = rc;
            S = h->S;
        }
        TimedPair tp;
        timed_begin(h, 1, tp);
        plain_update(kernel_law(&c), h->G, h->pp, h->P[h->cur], h->P[1 - h->cur], h->U0, h->U, h->F[0], h->F[1], h->F[2],
                     b[rk], rk, &h->st->dt, h->st, h->stream, S);
        timed_end(h, tp);
        h->launches++;
        h->cur = 1 - h->cur;
    }
}

static void enqueue_step(MaraGpuHandle* h)
{
    if (h->mixed) {
        mixed_set_timing(h->mixed, h->timing);
        mixed_enqueue_step(h->mixed, &h->st->dt, h->st, h->stream, nullptr);
        h->launches += mixed_launches_per_step(h->mixed);
    } else {
        enqueue_plain_step(h);
    }
}

static void enqueue_courant(MaraGpuHandle* h)
{
    launch_courant_init(h->st, h->stream);
    TimedPair tp;
    timed_begin(h, 2, tp);
    if (h->mixed) mixed_enqueue_courant(h->mixed, h->st, h->stream);
    else plain_courant(kernel_law(&h->cfg), h->G, h->pp, h->P[h->cur], h->st, h->stream);
    timed_end(h, tp);
    h->launches += 2;
}

// With the stream idle: the state's buffer parity from the steps that ran
// (the host flips its parity for every step it enqueues, also for steps that
// find the loop done and do no work), and the count reset.
static int settle_parity(MaraGpuHandle* h)
{
    const long long taken = h->st_host->taken;
    if (h->mixed) {
        mixed_sync_rotation(h->mixed, h->stream);
    } else {
        h->cur = (h->cur_base + (int) ((taken & 1) * (h->cfg.rk_order & 1))) & 1;
        h->cur_base = h->cur;
    }
    if (taken) {
        h->st_host->taken = 0;
        CK(cudaMemsetAsync(&h->st->taken, 0, sizeof(long long), h->stream));
    }
    return MARA_OK;
}

static int read_status(MaraGpuHandle* h)
{
    CK(cudaMemcpyAsync(h->st_host, h->st, sizeof(DevStatus), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    if (const int rs_ = settle_parity(h)) return rs_;
    const DevStatus& s = *h->st_host;
    int status = s.code;
    if (status == 0 && s.failures > 0) status = MARA_ERR_INVERSION_FAILURE;
    h->last_status = status;
    return status;
}

// Wait for the enqueued work and settle the state's buffer before reading it
// (download, diagnostics, Courant step): a status error is not a failure here.
static int sync_state(MaraGpuHandle* h)
{
    CK(cudaMemcpyAsync(h->st_host, h->st, sizeof(DevStatus), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return settle_parity(h);
}

static int clear_status(MaraGpuHandle* h)
{
    DevStatus z;
    std::memset(&z, 0, sizeof(z));
    z.first_zone = ~0ull;
    *h->st_host = z;
    CK(cudaMemcpyAsync(h->st, h->st_host, sizeof(DevStatus), cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return MARA_OK;
}

// configuration check and mesh description for mara_gpu_advance_noalloc
// (no_alloc.cu), which works without a handle
namespace mara {
int noalloc_validate(const MaraGpuConfig* c) { return validate(c); }
void noalloc_make_grid(const MaraGpuConfig* c, GridDesc* G) { make_grid(c, G); }
} // namespace mara

// ---------------------------------------------------------------------------
extern "C" {

int mara_gpu_create(const MaraGpuConfig* config, MaraGpuHandle** out)
{
    if (!config || !out) return MARA_ERR_ARGUMENT;
    *out = nullptr;
    int v = validate(config);
    if (v) return v;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return MARA_ERR_NO_DEVICE;
    if (config->device < 0 || config->device >= ndev) return MARA_ERR_NO_DEVICE;
    CK(cudaSetDevice(config->device));

    MaraGpuHandle* h = new (std::nothrow) MaraGpuHandle();
    if (!h) return MARA_ERR_ARGUMENT;
    h->cfg = *config;
    make_grid(config, &h->G);
    make_phys(config, &h->pp);
    int rc = MARA_OK;
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) { delete h; return MARA_ERR_CUDA; }
    if (cudaStreamCreateWithFlags(&h->aux, cudaStreamNonBlocking) != cudaSuccess) rc = MARA_ERR_CUDA;
    for (int e = 0; e < 17 && !rc; ++e)
        if (cudaEventCreateWithFlags(&h->ev[e], cudaEventDisableTiming) != cudaSuccess) rc = MARA_ERR_CUDA;
    if (cudaMallocHost((void**) &h->st_host, sizeof(DevStatus)) != cudaSuccess) rc = MARA_ERR_CUDA;
    const GridDesc& G = h->G;
    const size_t pbytes = sizeof(double) * (size_t) G.sP * G.nq;
    if (!rc) rc = alloc(h, (void**) &h->st, sizeof(DevStatus));
    if (!rc) rc = alloc(h, (void**) &h->stage_aos, pbytes);
    if (!rc && config->precision == MARA_PRECISION_FP64) {
        const size_t ubytes = sizeof(double) * (size_t) G.sU * G.nq;
        const size_t fbytes = sizeof(double) * (size_t) G.sF * G.nq;
        rc = alloc(h, (void**) &h->P[0], pbytes);
        if (!rc) rc = alloc(h, (void**) &h->P[1], pbytes);
        if (!rc) rc = alloc(h, (void**) &h->U0, ubytes);
        if (!rc) rc = alloc(h, (void**) &h->U, ubytes);
        for (int a = 0; a < 3 && !rc; ++a)
            if (G.n[a] > 1) rc = alloc(h, (void**) &h->F[a], fbytes);
    } else if (!rc) {
        rc = mixed_create(config, G, &h->mixed, h->stream, &h->bytes);
    }
    if (!rc) rc = clear_status(h);
    if (rc) { mara_gpu_destroy(h); return rc; }
    *out = h;
    return MARA_OK;
}

int mara_gpu_destroy(MaraGpuHandle* h)
{
    if (!h) return MARA_OK;
    cudaSetDevice(h->cfg.device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    for (auto& tp : h->timed) { cudaEventDestroy(tp.a); cudaEventDestroy(tp.b); }
    for (int g = 0; g < 2; ++g) if (h->graph[g]) cudaGraphExecDestroy(h->graph[g]);
    cudaFree(h->P[0]);
    cudaFree(h->P[1]);
    cudaFree(h->U0);
    cudaFree(h->U);
    for (int a = 0; a < 3; ++a) cudaFree(h->F[a]);
    cudaFree(h->stage_aos);
    cudaFree(h->st);
    cudaFree(h->diag);
    cudaFree(h->S);
    if (h->mixed) mixed_destroy(h->mixed);
    if (h->st_host) cudaFreeHost(h->st_host);
    for (int e = 0; e < 17; ++e) if (h->ev[e]) cudaEventDestroy(h->ev[e]);
    if (h->aux) cudaStreamDestroy(h->aux);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return MARA_OK;
}

// Transfers are split into chunks of whole cells: the copy of chunk k+1 (on
// the auxiliary stream) overlaps the layout conversion of chunk k (on the
// handle's stream).
static int chunks_of(const MaraGpuHandle* h)
{
    const size_t bytes = sizeof(double) * (size_t) h->G.sP * h->G.nq;
    if (bytes < (size_t(4) << 20)) return 1;
    return 8;
}

// The device address of a page-locked host array (cudaHostAlloc /
// cudaHostRegister), or null for pageable memory.  On this platform the GPU
// reaches page-locked host memory over the chip-to-chip link, so the layout
// conversion kernels can read or write the caller's array directly: the copy
// and the conversion are one pass, at the link's bandwidth.
static const void* direct_host_pointer(const void* p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

int mara_gpu_host_register(void* p, size_t bytes)
{
    if (!p || !bytes) return MARA_ERR_ARGUMENT;
    if (cudaHostRegister(p, bytes, cudaHostRegisterPortable | cudaHostRegisterMapped) != cudaSuccess) {
        cudaGetLastError();
        return MARA_ERR_CUDA;
    }
    return MARA_OK;
}

int mara_gpu_host_unregister(void* p)
{
    if (!p) return MARA_ERR_ARGUMENT;
    if (cudaHostUnregister(p) != cudaSuccess) {
        cudaGetLastError();
        return MARA_ERR_CUDA;
    }
    return MARA_OK;
}

int mara_gpu_upload(MaraGpuHandle* h, const double* P_aos)
{
    if (!h || !P_aos) return MARA_ERR_ARGUMENT;
    CK(cudaSetDevice(h->cfg.device));
    // a new state starts with a clean status (errors of the previous state
    // are reported until then)
    k_status_reset<<<1, 1, 0, h->stream>>>(h->st);
    h->launches++;
    h->cur_base = h->cur;   // the new state is written into P[cur]; the count of steps taken restarts
    if (h->mixed) mixed_load_begin(h->mixed, h->stream);
    if (const double* d = (const double*) direct_host_pointer(P_aos)) {
        const long long cells = h->G.sP;
        if (h->mixed) mixed_load_aos_range(h->mixed, d, 0, cells, h->st, h->stream);
        else launch_aos_to_soa_range(d, h->P[h->cur], h->G, 0, cells, h->stream);
        h->launches++;
        if (h->mixed) mixed_load_finish(h->mixed, h->st, h->stream);
        return cuda_status(cudaGetLastError());
    }
    const int C = chunks_of(h);
    const long long cells = h->G.sP, nq = h->G.nq;
    CK(cudaEventRecord(h->ev[16], h->stream));
    CK(cudaStreamWaitEvent(h->aux, h->ev[16], 0));
    for (int k = 0; k < C; ++k) {
        const long long c0 = cells * k / C, c1 = cells * (k + 1) / C;
        CK(cudaMemcpyAsync(h->stage_aos + c0 * nq, P_aos + c0 * nq, sizeof(double) * (c1 - c0) * nq,
                           cudaMemcpyHostToDevice, h->aux));
        CK(cudaEventRecord(h->ev[k], h->aux));
        CK(cudaStreamWaitEvent(h->stream, h->ev[k], 0));
        if (h->mixed) mixed_load_aos_range(h->mixed, h->stage_aos, c0, c1, h->st, h->stream);
        else launch_aos_to_soa_range(h->stage_aos, h->P[h->cur], h->G, c0, c1, h->stream);
        h->launches++;
    }
    if (h->mixed) mixed_load_finish(h->mixed, h->st, h->stream);
    return cuda_status(cudaGetLastError());
}

int mara_gpu_generate(MaraGpuHandle* h, const MaraInitialData* d)
{
    if (!h || !d) return MARA_ERR_ARGUMENT;
    if (d->kind < MARA_INIT_PLANAR_RIEMANN || d->kind > MARA_INIT_CYLINDER) return MARA_ERR_ARGUMENT;
    if (h->G.nq > 8) return MARA_ERR_CONFIG;  // the built-in states hold eight fields
    CK(cudaSetDevice(h->cfg.device));
    GenGeom geo;
    const int n[3] = {h->cfg.ni, h->cfg.nj, h->cfg.nk};
    for (int a = 0; a < 3; ++a) {
        geo.lower[a] = h->cfg.lower[a];
        geo.dx[a] = (h->cfg.upper[a] - h->cfg.lower[a]) / n[a];
    }
    const long long total = h->G.sP;
    k_generate<<<(unsigned) ((total + 255) / 256), 256, 0, h->stream>>>(h->stage_aos, h->G, geo, *d);
    k_status_reset<<<1, 1, 0, h->stream>>>(h->st);
    h->cur_base = h->cur;
    h->launches += 2;
    if (h->mixed) {
        mixed_load_begin(h->mixed, h->stream);
        mixed_load_aos_range(h->mixed, h->stage_aos, 0, total, h->st, h->stream);
        mixed_load_finish(h->mixed, h->st, h->stream);
    } else {
        launch_aos_to_soa_range(h->stage_aos, h->P[h->cur], h->G, 0, total, h->stream);
    }
    h->launches++;
    return cuda_status(cudaGetLastError());
}

int mara_gpu_assign_vector_potential(MaraGpuHandle* h, const double* A, double scale)
{
    if (!h || !A) return MARA_ERR_ARGUMENT;
    if (h->cfg.law != MARA_LAW_MHD && h->cfg.law != MARA_LAW_RMHD) return MARA_ERR_CONFIG;
    CK(cudaSetDevice(h->cfg.device));
    if (const int rs_ = sync_state(h)) return rs_;
    const VecPot shape{nullptr, h->G.N[0] + 1, h->G.N[1] + 1, h->G.N[2] + 1};
    const size_t abytes = sizeof(double) * 9 * (size_t) shape.f0 * shape.f1 * shape.f2;
    double* dA = nullptr;
    CK(cudaMallocAsync(&dA, abytes, h->stream));
    int rc = cuda_status(cudaMemcpyAsync(dA, A, abytes, cudaMemcpyHostToDevice, h->stream));
    const long long total = h->G.sP;
    if (rc == MARA_OK) {
        // the resident state as FP64 primitives with guards, the field
        // replaced, then loaded back like an upload
        if (h->mixed) mixed_store_aos_range(h->mixed, h->stage_aos, 0, total, h->stream);
        else launch_soa_to_aos_range(h->P[h->cur], h->stage_aos, h->G, 0, total, h->stream);
        VecPot V = shape;
        V.A = dA;
        k_assign_b<<<(unsigned) ((total + 255) / 256), 256, 0, h->stream>>>(h->stage_aos, h->G, V, scale);
        k_status_reset<<<1, 1, 0, h->stream>>>(h->st);
        h->cur_base = h->cur;
        if (h->mixed) {
            mixed_load_begin(h->mixed, h->stream);
            mixed_load_aos_range(h->mixed, h->stage_aos, 0, total, h->st, h->stream);
            mixed_load_finish(h->mixed, h->st, h->stream);
        } else {
            launch_aos_to_soa_range(h->stage_aos, h->P[h->cur], h->G, 0, total, h->stream);
        }
        h->launches += 4;
        rc = cuda_status(cudaGetLastError());
    }
    const int rf = cuda_status(cudaFreeAsync(dA, h->stream));
    if (rc == MARA_OK) rc = cuda_status(cudaStreamSynchronize(h->stream));
    return rc != MARA_OK ? rc : rf;
}

int mara_gpu_download(MaraGpuHandle* h, double* P_aos)
{
    if (!h || !P_aos) return MARA_ERR_ARGUMENT;
    CK(cudaSetDevice(h->cfg.device));
    if (const int rs_ = sync_state(h)) return rs_;
    if (double* d = (double*) direct_host_pointer(P_aos)) {
        const long long cells = h->G.sP;
        if (h->mixed) mixed_store_aos_range(h->mixed, d, 0, cells, h->stream);
        else launch_soa_to_aos_range(h->P[h->cur], d, h->G, 0, cells, h->stream);
        h->launches++;
        CK(cudaStreamSynchronize(h->stream));
        return cuda_status(cudaGetLastError());
    }
    const int C = chunks_of(h);
    const long long cells = h->G.sP, nq = h->G.nq;
    for (int k = 0; k < C; ++k) {
        const long long c0 = cells * k / C, c1 = cells * (k + 1) / C;
        if (h->mixed) mixed_store_aos_range(h->mixed, h->stage_aos, c0, c1, h->stream);
        else launch_soa_to_aos_range(h->P[h->cur], h->stage_aos, h->G, c0, c1, h->stream);
        h->launches++;
        CK(cudaEventRecord(h->ev[k], h->stream));
        CK(cudaStreamWaitEvent(h->aux, h->ev[k], 0));
        CK(cudaMemcpyAsync(P_aos + c0 * nq, h->stage_aos + c0 * nq, sizeof(double) * (c1 - c0) * nq,
                           cudaMemcpyDeviceToHost, h->aux));
    }
    CK(cudaEventRecord(h->ev[16], h->aux));
    CK(cudaStreamWaitEvent(h->stream, h->ev[16], 0));
    CK(cudaStreamSynchronize(h->stream));
    return MARA_OK;
}

int mara_gpu_advance(MaraGpuHandle* h, double t0, double dt)
{
    (void) t0;
    if (!h) return MARA_ERR_ARGUMENT;
    CK(cudaSetDevice(h->cfg.device));
    if (h->mixed) mixed_set_timing(h->mixed, h->timing);
    if (h->mixed && mixed_enqueue_advance(h->mixed, dt, h->st, h->stream)) {
        h->launches += mixed_launches_per_step(h->mixed);
    } else {
        launch_set_dt(h->st, dt, h->stream);
        h->launches++;
        enqueue_step(h);
        if (const int se = take_source_error(h)) return se;
        k_step_taken<<<1, 1, 0, h->stream>>>(h->st);
        h->launches++;
    }
    h->steps++;
    return cuda_status(cudaGetLastError());
}

int mara_gpu_advance_host(MaraGpuHandle* h, double* P_aos, double t0, double dt)
{
    if (h && P_aos && h->mixed && !h->timing && mixed_host_step_capable(h->mixed)) {
        if (double* d = (double*) direct_host_pointer(P_aos)) {
            // page-locked host array: transfers and stages pipelined in one launch
            CK(cudaSetDevice(h->cfg.device));
            k_status_reset<<<1, 1, 0, h->stream>>>(h->st);
            h->launches++;
            const int rc = mixed_advance_host_step(h->mixed, d, dt, h->st, h->stream, &h->launches);
            if (rc != MIXED_NOT_TAKEN) {
                if (rc) return rc;
                h->steps++;
                return read_status(h);
            }
            // not available on this device: the unpipelined path below
        }
    }
    int rc = mara_gpu_upload(h, P_aos);
    if (!rc) rc = mara_gpu_advance(h, t0, dt);
    if (!rc) rc = mara_gpu_download(h, P_aos);
    if (!rc) rc = read_status(h);
    return rc;
}

int mara_gpu_courant(MaraGpuHandle* h, double* dt)
{
    if (!h || !dt) return MARA_ERR_ARGUMENT;
    CK(cudaSetDevice(h->cfg.device));
    if (const int rs_ = sync_state(h)) return rs_;
    enqueue_courant(h);
    const int rc = read_status(h);
    *dt = __builtin_bit_cast(double, h->st_host->dt_bits);
    return rc;
}

// steps per launch of the cluster form (a few ms of work at most)
constexpr int CLUSTER_STEPS = 1024;

// one driver-loop step: Courant step, dt, the RK stages, the clock
static void enqueue_run_step(MaraGpuHandle* h, double cfl, double t_final)
{
    if (h->mixed) mixed_set_timing(h->mixed, h->timing);
    if (h->mixed && mixed_enqueue_run_step(h->mixed, cfl, t_final, h->st, h->stream)) {
        h->launches += mixed_launches_per_step(h->mixed);
        return;
    }
    enqueue_courant(h);
    launch_dt_from_courant(h->st, cfl, t_final, h->stream);
    enqueue_step(h);
    launch_advance_time(h->st, h->stream);
    h->launches += 2;
}

static int build_run_graph(MaraGpuHandle* h, int which, double cfl, double t_final)
{
    cudaGraph_t g;
    const int timing = h->timing;
    h->timing = 0;
    const int64_t launches = h->launches;
    CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    enqueue_run_step(h, cfl, t_final);
    CK(cudaStreamEndCapture(h->stream, &g));
    if (const int se = take_source_error(h)) {
        cudaGraphDestroy(g);
        h->timing = timing;
        h->launches = launches;
        return se;
    }
    h->timing = timing;
    h->launches = launches;
    if (h->graph[which]) cudaGraphExecDestroy(h->graph[which]);
    const cudaError_t e = cudaGraphInstantiate(&h->graph[which], g, 0);
    cudaGraphDestroy(g);
    return cuda_status(e);
}

static int launches_per_run_step(MaraGpuHandle* h)
{
    if (h->mixed && mixed_fused(h->mixed)) return mixed_launches_per_step(h->mixed);
    int n = 2 /* courant init + courant */ + 2 /* dt, time */;
    if (h->mixed) return n + mixed_launches_per_step(h->mixed);
    for (int a = 0; a < 3; ++a) if (h->G.n[a] > 1) n += h->cfg.rk_order;
    return n + h->cfg.rk_order;
}

static int enqueue_run(MaraGpuHandle* h, int max_steps, double cfl, double t_final)
{
    if (h->mixed && !h->timing && mixed_cluster_capable(h->mixed)) {
        // a small 1-D grid: chunks of steps, each one launch on a cluster
        for (int left = max_steps; left > 0; left -= CLUSTER_STEPS) {
            const int k = left < CLUSTER_STEPS ? left : CLUSTER_STEPS;
            const int rc = mixed_enqueue_cluster_steps(h->mixed, k, cfl, t_final, h->st, h->stream);
            if (rc) return rc;
            h->steps += k;
            h->launches++;
        }
        return cuda_status(cudaGetLastError());
    }
    const bool use_graph = !h->timing;
    if (use_graph && (h->graph_cfl != cfl || h->graph_tfinal != t_final)) {
        for (int g = 0; g < 2; ++g) if (h->graph[g]) { cudaGraphExecDestroy(h->graph[g]); h->graph[g] = nullptr; }
        h->graph_cfl = cfl;
        h->graph_tfinal = t_final;
    }
    for (int n = 0; n < max_steps; ++n) {
        if (use_graph) {
            // the P ping-pong parity decides which of two captured graphs applies
            const int which = h->mixed ? mixed_parity(h->mixed) : h->cur;
            if (!h->graph[which]) {
                const int cur0 = h->cur;
                const int par0 = h->mixed ? mixed_parity(h->mixed) : 0;
                int rc = build_run_graph(h, which, cfl, t_final);
                h->cur = cur0;
                if (h->mixed) mixed_set_parity(h->mixed, par0);
                if (rc) return rc;
            }
            CK(cudaGraphLaunch(h->graph[which], h->stream));
            // advance the host-side parity exactly as the captured step did
            if (h->mixed) mixed_advance_parity(h->mixed);
            else h->cur = (h->cur + h->cfg.rk_order) & 1;
            h->launches += launches_per_run_step(h);
        } else {
            enqueue_run_step(h, cfl, t_final);
            if (const int se = take_source_error(h)) return se;
        }
        h->steps++;
    }
    return cuda_status(cudaGetLastError());
}

int mara_gpu_run(MaraGpuHandle* h, int max_steps, double cfl, double t_final, double* t, int* steps_done)
{
    if (!h || !t) return MARA_ERR_ARGUMENT;
    CK(cudaSetDevice(h->cfg.device));
    k_run_begin<<<1, 1, 0, h->stream>>>(h->st, *t);
    h->launches++;
    // with an end time, look at the device's done flag every 64 steps so the
    // host stops enqueuing once the run has reached t_final
    const int chunk = t_final >= 0.0 ? 64 : max_steps;
    int rc = MARA_OK;
    for (int left = max_steps; left > 0 && rc == MARA_OK; left -= chunk) {
        rc = enqueue_run(h, left < chunk ? left : chunk, cfl, t_final);
        if (rc || left <= chunk || t_final < 0.0) break;
        rc = read_status(h);
        if (rc || h->st_host->done) break;
    }
    if (rc) return rc;
    rc = read_status(h);
    *t = h->st_host->t;
    if (steps_done) *steps_done = (int) h->st_host->steps;
    return rc;
}

int mara_gpu_run_async(MaraGpuHandle* h, int max_steps, double cfl, double t_final)
{
    if (!h) return MARA_ERR_ARGUMENT;
    CK(cudaSetDevice(h->cfg.device));
    return enqueue_run(h, max_steps, cfl, t_final);
}

int mara_gpu_synchronize(MaraGpuHandle* h)
{
    if (!h) return MARA_ERR_ARGUMENT;
    CK(cudaSetDevice(h->cfg.device));
    return read_status(h);
}

int mara_gpu_stats(MaraGpuHandle* h, MaraGpuStats* s)
{
    if (!h || !s) return MARA_ERR_ARGUMENT;
    const int rc = read_status(h);
    const DevStatus& d = *h->st_host;
    std::memset(s, 0, sizeof(*s));
    s->status = rc;
    s->failures = d.failures;
    if (d.failures > 0 && d.first_zone != ~0ull) {
        const unsigned long long z = d.first_zone;
        const int n0 = h->G.n[0], n1 = h->G.n[1];
        s->first_zone[0] = (int) (z % n0);
        s->first_zone[1] = (int) ((z / n0) % n1);
        s->first_zone[2] = (int) (z / ((unsigned long long) n0 * n1));
        s->first_code = d.first_code;
    }
    s->steps = h->steps;
    s->kernel_launches = h->launches;
    s->last_dt = d.dt;
    return MARA_OK;
}

void* mara_gpu_stream(MaraGpuHandle* h) { return h ? (void*) h->stream : nullptr; }

int mara_gpu_set_kernel_timing(MaraGpuHandle* h, int enable)
{
    if (!h) return MARA_ERR_ARGUMENT;
    h->timing = enable ? 1 : 0;
    return MARA_OK;
}

int mara_gpu_kernel_times(MaraGpuHandle* h, double ms_total[3], int64_t launches[3])
{
    if (!h) return MARA_ERR_ARGUMENT;
    CK(cudaStreamSynchronize(h->stream));
    for (auto& tp : h->timed) {
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, tp.a, tp.b);
        h->ms_total[tp.cls] += ms;
        h->timed_launches[tp.cls] += 1;
        cudaEventDestroy(tp.a);
        cudaEventDestroy(tp.b);
    }
    h->timed.clear();
    if (h->mixed) mixed_kernel_times(h->mixed, h->ms_total, h->timed_launches);
    for (int c = 0; c < 3; ++c) {
        if (ms_total) ms_total[c] = h->ms_total[c];
        if (launches) launches[c] = h->timed_launches[c];
        h->ms_total[c] = 0;
        h->timed_launches[c] = 0;
    }
    return MARA_OK;
}

int mara_gpu_monopole(MaraGpuHandle* h, double mesh_spacing, double* max_abs)
{
    if (!h || !max_abs || !(mesh_spacing > 0.0)) return MARA_ERR_ARGUMENT;
    if (h->cfg.law == MARA_LAW_HYDRO) return MARA_ERR_CONFIG;
    CK(cudaSetDevice(h->cfg.device));
    if (const int rs_ = sync_state(h)) return rs_;
    const void* P = h->mixed ? (const void*) mixed_primitives(h->mixed) : (const void*) h->P[h->cur];
    if (!P) return MARA_ERR_CONFIG;
    unsigned long long* out = &h->st->dt_bits;  // scratch word: the next Courant call re-initialises it
    CK(cudaMemsetAsync(out, 0, sizeof(unsigned long long), h->stream));
    launch_monopole_max(P, h->mixed != nullptr, h->G, mesh_spacing, out, h->stream);
    h->launches++;
    unsigned long long bits = 0;
    CK(cudaMemcpyAsync(&bits, out, sizeof(bits), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    *max_abs = __builtin_bit_cast(double, bits);
    return MARA_OK;
}

int mara_gpu_set_source_terms(MaraGpuHandle* h, MaraSourceTermsFn fn, void* user)
{
    if (!h) return MARA_ERR_ARGUMENT;
    if (h->mixed) return fn ? MARA_ERR_CONFIG : MARA_OK;
    CK(cudaSetDevice(h->cfg.device));
    if (fn && !h->S) {
        const size_t bytes = (size_t) h->G.sP * h->G.nq * sizeof(double);
        if (alloc(h, (void**) &h->S, bytes)) return MARA_ERR_CUDA;
    }
    h->src_fn = fn;
    h->src_user = user;
    h->src_error = MARA_OK;
    // the captured step graphs hold what the previous function enqueued
    for (int g = 0; g < 2; ++g)
        if (h->graph[g]) { cudaGraphExecDestroy(h->graph[g]); h->graph[g] = nullptr; }
    return MARA_OK;
}

int mara_gpu_num_diagnostics(const MaraGpuHandle* h)
{
    if (!h) return 0;
    return h->cfg.law == MARA_LAW_HYDRO ? 5 : kernel_law(&h->cfg) == LAW_MHD_COOL ? 18 : 17;
}

int mara_gpu_volume_diagnostics(MaraGpuHandle* h, double* D, int* count)
{
    if (!h || !D) return MARA_ERR_ARGUMENT;
    CK(cudaSetDevice(h->cfg.device));
    if (const int rs_ = sync_state(h)) return rs_;
    const size_t nd = DIAG_MAX;
    const size_t doubles = (size_t) DIAG_BLOCKS * nd + nd + 1;  // partials, totals, error word
    if (!h->diag) {
        if (alloc(h, (void**) &h->diag, doubles * sizeof(double))) return MARA_ERR_CUDA;
    }
    double* partial = h->diag;
    double* out = h->diag + (size_t) DIAG_BLOCKS * nd;
    int* err = (int*) (out + nd);
    CK(cudaMemsetAsync(err, 0, sizeof(int), h->stream));
    if (h->mixed) mixed_volume_diagnostics(h->mixed, partial, err, out, h->stream);
    else launch_volume_diag_plain(kernel_law(&h->cfg), h->P[h->cur], h->G, h->pp, partial, err, out, h->stream);
    h->launches += 3;
    const int n = mara_gpu_num_diagnostics(h);
    double host[DIAG_MAX + 1];
    CK(cudaMemcpyAsync(host, out, sizeof(double) * (nd + 1), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    int e = 0;
    std::memcpy(&e, &host[nd], sizeof(int));
    if (e) return e;
    for (int q = 0; q < n; ++q) D[q] = host[q];
    if (count) *count = n;
    return MARA_OK;
}

int mara_gpu_field_diagnostics(MaraGpuHandle* h, double mesh_spacing, double* out_aos)
{
    if (!h || !out_aos || !(mesh_spacing > 0.0)) return MARA_ERR_ARGUMENT;
    if (h->cfg.law == MARA_LAW_HYDRO) return MARA_ERR_CONFIG;
    CK(cudaSetDevice(h->cfg.device));
    if (const int rs_ = sync_state(h)) return rs_;
    const void* P = h->mixed ? (const void*) mixed_primitives(h->mixed) : (const void*) h->P[h->cur];
    if (!P) return MARA_ERR_CONFIG;
    const size_t bytes = (size_t) h->G.N[0] * h->G.N[1] * h->G.N[2] * 4 * sizeof(double);
    double* d = nullptr;
    CK(cudaMallocAsync((void**) &d, bytes, h->stream));
    launch_field_diag(P, h->mixed != nullptr, h->G, mesh_spacing, d, h->stream);
    h->launches++;
    const cudaError_t e = cudaMemcpyAsync(out_aos, d, bytes, cudaMemcpyDeviceToHost, h->stream);
    cudaFreeAsync(d, h->stream);
    CK(e);
    CK(cudaStreamSynchronize(h->stream));
    return MARA_OK;
}

int64_t mara_gpu_device_bytes(const MaraGpuHandle* h) { return h ? h->bytes : 0; }

const char* mara_gpu_status_string(int s)
{
    switch (s) {
        case MARA_OK: return "success";
        case MARA_C2P_CONS_CONTAINS_NAN: return "input conserved state contained nan's";
        case MARA_C2P_CONS_NEGATIVE_DENSITY: return "input conserved state has negative density";
        case MARA_C2P_CONS_NEGATIVE_ENERGY: return "input conserved state has negative energy";
        case MARA_C2P_PRIM_CONTAINS_NAN: return "derived primitive state contains nan's";
        case MARA_C2P_PRIM_NEGATIVE_PRESSURE: return "derived primitive state has negative pressure";
        case MARA_C2P_PRIM_NEGATIVE_RESTMASS: return "derived primitive state contains negative density";
        case MARA_C2P_PRIM_SUPERLUMINAL: return "derived primitive state contains superluminal velocity";
        case MARA_C2P_MAXITER: return "rootfinder hit maximum iterations";
        case MARA_ERR_INVERSION_FAILURE: return "primitive variable inversion failed in one or more zones";
        case MARA_ERR_SUPERLUMINAL: return "got superluminal velocity";
        case MARA_ERR_BAD_EIGENVALUES: return "got bad eigenvalues";
        case MARA_ERR_GUARD_TOO_SMALL: return "Boundary region of mesh data is smaller than the scheme's stencil";
        case MARA_ERR_CONFIG: return "invalid configuration";
        case MARA_ERR_CUDA: return "a CUDA runtime call failed";
        case MARA_ERR_NO_DEVICE: return "no CUDA device";
        case MARA_ERR_ARGUMENT: return "invalid argument";
        case MARA_ERR_TOO_LARGE: return "size exceeds the supported maximum";
        default: return "unknown status";
    }
}

} // extern "C"
