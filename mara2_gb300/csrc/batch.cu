// batch.cu -- many independent hydro grids advanced together (include/
// mara_batch.h).
//
// Device tables, one entry per slot: HGrid (state pointers, shape, bc,
// gamma), the driver state (t, dt, t_final, cfl factor, done, steps, Courant
// bits) and the buffer rotation.  Two tile lists (1-D tiles, 2-D tiles) cover
// every resident grid.  Two launch forms, with the same arithmetic and bits:
// (stage form) each RK stage is two launches of the fused stage kernel
// (hydro_tile.cuh), one per list, whose CTAs stride over the list whatever
// mix of grids is resident, and a batch step -- per-grid dt, the RK stages,
// the per-grid Courant reduction fused into the last stage, the time update
// -- is captured once as a CUDA graph; (persistent form) every stage of a
// batch step over both lists in one cooperative launch with grid-wide
// barriers between the stages (batch_step_kernel).  Admitting or retiring a
// grid rewrites the tables and the tile lists (device-resident counts),
// never the graph or the launch.
//
// Memory: each grid holds its FP32-pair state (2 rotation buffers for RK1/2,
// 3 for RK3) allocated stream-ordered from the device's memory pool and
// counted against the batch's HBM budget; admission fails with
// MARA_ERR_NO_ROOM when the budget or the slot table is full.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/mara_batch.h"
#include "hydro_cluster.cuh"
#include "hydro_tile.cuh"

namespace mara {

struct SlotHost {
    bool used = false;
    bool finished_reported = false;
    int dims = 0, n0 = 0, n1 = 1, g0 = 0, g1 = 0;
    int bc = 0;
    double gamma = 5. / 3;
    int64_t bytes = 0;
    float* bufs[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    int64_t zones = 0;
    bool cluster = false;   // advanced on its own thread-block cluster (a small 1-D grid with an end time)
    int bucket = 0;         // its zones-per-CTA class
};

// Small 1-D grids with an end time run their driver loop on thread-block
// clusters (hydro_cluster.cuh) launched on side streams, K steps per batch
// step call, instead of stepping in lockstep with the tile lists: a 1-D
// request can need a hundred times the steps of the 2-D ones, and in
// lockstep each of its steps would cost a whole batch step.  All clusters
// of one launch have the same size, and every CTA the shared memory of the
// launch's largest grid, so the grids are grouped in classes of (CTAs per
// cluster, most zones per CTA): a grid of n zones takes the largest
// power-of-two C <= n / 128 (1 to 8), and ceil(n / C) zones per CTA.  The
// arithmetic of a zone does not depend on C.
constexpr int CLUSTER_BUCKETS = 6;
static const int CLUSTER_BUCKET_C[CLUSTER_BUCKETS] = {1, 2, 4, 8, 8, 8};
static const int CLUSTER_BUCKET_M[CLUSTER_BUCKETS] = {256, 256, 256, 256, 512, 1024};
constexpr int CLUSTER_MAX_ZONES = 8 * 1024;
constexpr int CLUSTER_RUNNING = 3;  // done[] of a slot its cluster advances

static int cluster_bucket(int n)
{
    if (n < 256) return 0;
    if (n < 512) return 1;
    if (n < 1024) return 2;
    const int m = (n + 7) / 8;
    return m <= 256 ? 3 : m <= 512 ? 4 : 5;
}

__global__ void k_slot_init(HGrid* grids, int* rot, double* t, double* dt, double* tfin, double* cflp, int* done,
                            long long* steps, int* pend, int slot, HGrid g, double t_final, double cfl, int done0)
{
    grids[slot] = g;
    rot[slot] = 0;
    t[slot] = 0.0;
    dt[slot] = 0.0;
    tfin[slot] = t_final;
    cflp[slot] = cfl;
    done[slot] = done0;
    steps[slot] = 0;
    pend[slot] = 0;
}

__global__ void k_slot_clear(int* done, int slot) { done[slot] = 1; }

// Start of a batch step, one thread per slot: the previous step's clock
// advance (t += dt, the step count, the RK1 buffer swap), then the drivers'
// dt = min(cfl * courant, t_final - t) (src/Problems.cpp:181-186) from the
// Courant step the previous step's last stage (or the load) reduced, and the
// reduction slot reset for this step's last stage.  A grid whose t has
// reached t_final stops (done = 2) with its state as after its last step.
__global__ void k_batch_begin(int n, unsigned long long* cflbits, const double* cflp, double* t, const double* tfin,
                              double* dt, int* done, long long* steps, int* rot, int* pend, int flip)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n || done[s]) return;
    if (pend[s]) {
        t[s] += dt[s];
        steps[s] += 1;
        if (flip) rot[s] ^= 1;
        pend[s] = 0;
    }
    if (!(t[s] < tfin[s])) { done[s] = 2; return; }   // 2: finished (1: empty slot)
    const double courant = __longlong_as_double((long long) cflbits[s]);
    double d = cflp[s] * courant;
    const double d2 = tfin[s] - t[s];
    dt[s] = d < d2 ? d : d2;
    cflbits[s] = (unsigned long long) __double_as_longlong(DBL_MAX);
    pend[s] = 1;
}

__global__ void k_set_int(int* p, int v) { *p = v; }
__global__ void k_set_u64(unsigned long long* p, unsigned long long v) { *p = v; }

// host FP64 primitives (AoS with guards) -> FP32-pair conserved state of one
// slot, and the grid's first Courant step
__global__ void k_batch_load(const double* __restrict__ aos, HGrid g, int g0, int g1, int N0, int N1, double inv_gm1,
                             unsigned long long* cflbit)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    float zdt = 3.0e38f;
    if (x < g.n0) {
        const long long c = (long long) (x + g0) * N1 + (y + g1);  // AoS cell (i, j), k = 0
        double P[5], U[5];
#pragma unroll
        for (int q = 0; q < 5; ++q) P[q] = aos[c * 5 + q];
        hydro_p2u_d(P, inv_gm1, U);
        const long long o = (long long) y * g.n0 + x;
        float Uf[5];
#pragma unroll
        for (int q = 0; q < 5; ++q) {
            const df d = df_from_double(U[q]);
            g.Uh[0][q * g.sU + o] = d.hi;
            g.Ul[0][q * g.sU + o] = d.lo;
            Uf[q] = d.hi;
        }
        zdt = hydro_zone_dt(g.gamma, g.lmin, Uf);
    }
    block_min_to(cflbit, zdt);
}

// FP32-pair state -> FP64 primitives (AoS with guards; guards are boundary
// images of interior zones)
__global__ void k_batch_store(HGrid g, int buf, int g0, int g1, int N0, int N1, double gamma, double* __restrict__ aos)
{
    const long long c = blockIdx.x * (long long) blockDim.x + threadIdx.x;
    if (c >= (long long) N0 * N1) return;
    const int j = (int) (c % N1), i = (int) (c / N1);
    int fx = 0, fy = 0;
    const int x = bc_image(i - g0, g.n0, g.bc, fx);
    const int y = g.n1 > 1 ? bc_image(j - g1, g.n1, g.bc, fy) : 0;
    const long long o = (long long) y * g.n0 + x;
    double U[5];
#pragma unroll
    for (int q = 0; q < 5; ++q) U[q] = f2d_exact(g.Uh[buf][q * g.sU + o]) + f2d_exact(g.Ul[buf][q * g.sU + o]);
    double P[5];
    hydro_u2p_d(U, gamma - 1.0, P);
    if (fx) P[1] = -P[1];
    if (fy) P[2] = -P[2];
#pragma unroll
    for (int q = 0; q < 5; ++q) aos[c * 5 + q] = P[q];
}

// ---- the persistent step ----------------------------------------------------------
// Every RK stage of every grid in the tile lists for one batch step, in one
// cooperative launch: the step start of every slot (k_batch_begin's
// arithmetic), a grid-wide barrier, then per stage the CTAs stride over the
// 1-D and the 2-D tiles together (MASK: which lists the kernel serves), a
// barrier between stages.  CTAs read what other CTAs of the launch wrote:
// the per-slot scalars (dt, the buffer rotation, done) through L2
// (ld.global.cg), and a stage's input, which the previous stage wrote, with
// ordinary loads - no SM has read those lines earlier in the launch (stage
// k reads rotation buffer k, which only stage k - 1 wrote, and U0, which no
// stage before the last writes), so its L1 holds no stale copy, and the
// kernel boundary orders one step's writes before the next step's reads.
// The arithmetic is the tile kernels' (tile_stage), so a grid gives the same
// bits as with one launch per stage.
struct BatchArgs {
    const HGrid* grids;
    const TileRef* tiles1;
    const TileRef* tiles2;
    const int* ntiles;               // device-resident counts: [0] 1-D, [1] 2-D
    int* rot;
    double* t;
    double* dt;
    const double* tfin;
    const double* cflp;
    int* done;
    int* pend;
    long long* steps;
    unsigned long long* cflbits;
    unsigned* bar;                   // [0] arrivals, [1] generation
    int* err;                        // set when a barrier wait gave up
    int nslots, order, flip;
    float b[3];
};

constexpr int BATCH_POLLS = 1 << 24;  // a few seconds of waiting at a barrier, then an error

// Grid-wide barrier of a cooperative launch (all CTAs resident): one thread
// per CTA arrives on a counter; the last arrival resets it and bumps the
// generation the others wait on.  Every wait is bounded: past the limit the
// waiting CTA sets the error flag and returns false, as do CTAs that find the
// flag set, so the launch ends and the host reads the error.
__device__ __forceinline__ bool grid_barrier(const BatchArgs& A)
{
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        ok = 1;
        volatile unsigned* gen = A.bar + 1;
        const unsigned g = *gen;
        __threadfence();
        if (atomicAdd(A.bar, 1u) == gridDim.x - 1) {
            atomicExch(A.bar, 0u);
            __threadfence();
            atomicAdd(A.bar + 1, 1u);
        } else {
            int polls = 0;
            while (*gen == g) {
                if (*(volatile int*) A.err) { ok = 0; break; }
                if (++polls > BATCH_POLLS) { atomicExch(A.err, 1); ok = 0; break; }
                __nanosleep(polls < 64 ? 32 : 256);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return ok != 0;
}

// k_batch_begin for one slot, its operands read from L2
__device__ __forceinline__ void batch_begin_slot(const BatchArgs& A, int s)
{
    if (__ldcg(A.done + s)) return;
    if (__ldcg(A.pend + s)) {
        A.t[s] = __ldcg(A.t + s) + __ldcg(A.dt + s);
        A.steps[s] = __ldcg(A.steps + s) + 1;
        if (A.flip) A.rot[s] = __ldcg(A.rot + s) ^ 1;
        A.pend[s] = 0;
    }
    const double t = __ldcg(A.t + s), tf = __ldcg(A.tfin + s);
    if (!(t < tf)) { A.done[s] = 2; return; }   // 2: finished (1: empty slot)
    const double courant = __longlong_as_double((long long) __ldcg(A.cflbits + s));
    double d = __ldcg(A.cflp + s) * courant;
    const double d2 = tf - t;
    A.dt[s] = d < d2 ? d : d2;
    A.cflbits[s] = (unsigned long long) __double_as_longlong(DBL_MAX);
    A.pend[s] = 1;
}

template <int RECON, int RIEMANN, int T1, int TY2, int MASK>
__global__ void __launch_bounds__(256, 4) batch_step_kernel(const __grid_constant__ BatchArgs A)
{
    __shared__ union {
        TileSmem<1, RECON, T1, 1> s1;
        TileSmem<2, RECON, 32, TY2> s2;
    } sm;
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x, gstride = gridDim.x * blockDim.x;
    for (int s = gtid; s < A.nslots; s += gstride) batch_begin_slot(A, s);
    if (!grid_barrier(A)) return;
    const int n1 = MASK & 1 ? __ldcg(A.ntiles) : 0, n2 = MASK & 2 ? __ldcg(A.ntiles + 1) : 0;
    for (int rk = 0; rk < A.order; ++rk) {
        const int last = rk == A.order - 1;
        const float b = A.b[rk];
        for (int w = blockIdx.x; w < n1 + n2; w += gridDim.x) {
            const bool one = w < n1;
            const TileRef tr = one ? A.tiles1[w] : A.tiles2[w - n1];
            if (__ldcg(A.done + tr.grid)) continue;   // the same for the whole CTA
            struct {
                const double* dtp;
                unsigned long long* slot;
                __device__ float dt() const { return (float) __ldcg(dtp); }
                __device__ bool proceed() const { return true; }
                __device__ unsigned long long* cfl() const { return slot; }
            } at{A.dt + tr.grid, A.cflbits + tr.grid};
            const int r = __ldcg(A.rot + tr.grid);
            if constexpr ((MASK & 1) != 0) {
                if (one) {
                    tile_stage<1, RECON, RIEMANN, T1, 1, 256, false>(sm.s1, A.grids[tr.grid], tr, r, rk, b, 1.f - b,
                                                                     last, at);
                    continue;
                }
            }
            if constexpr ((MASK & 2) != 0)
                tile_stage<2, RECON, RIEMANN, 32, TY2, 256, false, false, false, true>(sm.s2, A.grids[tr.grid], tr, r,
                                                                                    rk, b, 1.f - b, last, at);
        }
        // the last stage's Courant reductions are read by the next launch
        if (!last && !grid_barrier(A)) return;
    }
}

} // namespace mara

using namespace mara;

struct MaraBatch {
    MaraBatchConfig cfg;
    cudaStream_t stream = nullptr;
    int sms = 0;
    int nslots = 0;
    // device tables
    HGrid* grids = nullptr;
    int* rot = nullptr;
    double *t = nullptr, *dt = nullptr, *tfin = nullptr, *cflp = nullptr;
    int* done = nullptr;
    int* pend = nullptr;    // a step was taken whose clock advance the next step start applies
    long long* steps = nullptr;
    unsigned long long* cflbits = nullptr;
    TileRef* tiles[2] = {nullptr, nullptr};
    int* ntiles = nullptr;  // [0] 1-D, [1] 2-D
    int max_tiles[2] = {0, 0};
    // host
    std::vector<SlotHost> slots;
    std::vector<int> done_host;
    TileRef* tiles_host[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};  // pinned, double-buffered
    cudaEvent_t tiles_ev[2] = {nullptr, nullptr};
    int tiles_buf = 0;
    bool dirty = true;
    double* staging = nullptr;
    int64_t staging_elems = 0;
    int64_t bytes_in_use = 0;
    int64_t zone_updates = 0;
    int64_t step_count = 0;
    int64_t launches = 0;
    int tile1 = 256, tile2 = 2;
    int ctas[2] = {0, 0};
    int count[2] = {0, 0};  // tiles in each list (host copy)
    // cluster slots: per class, the device list, its pinned staging
    // (double-buffered with the tile lists) and count; side streams; round
    // events (main stream start and graph end, each class's end); steps per
    // round of the cluster slots, adapted to the main stream's round time
    bool clusters = true;
    int* cl_slots[CLUSTER_BUCKETS] = {};
    int* cl_host[CLUSTER_BUCKETS][2] = {};
    int cl_count[CLUSTER_BUCKETS] = {};
    cudaStream_t side[CLUSTER_BUCKETS] = {};
    cudaEvent_t ev_start = nullptr, ev_main_end = nullptr;
    cudaEvent_t ev_side_end[CLUSTER_BUCKETS] = {};
    bool round_open = false;   // a round's events await reading
    int round_mask = 0;        // the tile lists that round launched
    bool round_side[CLUSTER_BUCKETS] = {};
    int cl_steps[CLUSTER_BUCKETS] = {};
    // one captured step per combination of non-empty tile lists (bit 0: 1-D,
    // bit 1: 2-D), so that a step launches only the lists that hold tiles
    cudaGraphExec_t graph[4] = {nullptr, nullptr, nullptr, nullptr};
    // the persistent form: one cooperative launch per mara_batch_step call
    bool persistent = false;
    int pgrid[4] = {0, 0, 0, 0};  // its CTAs by tile-list mask (SMs x CTAs per SM)
    unsigned* bar = nullptr; // grid barrier: arrivals, generation
    int* kerr = nullptr;     // set by a barrier wait that gave up
};

typedef void (*TileKernel)(const HGrid*, const TileRef*, const int*, const int*, const double*, int, const int*, int,
                           int, float, float, int, unsigned long long*, int, int);

template <int RECON, int RIEMANN>
static TileKernel pick_1d(int tile)
{
    switch (tile) {
        case 128: return hydro_tile_kernel<1, RECON, RIEMANN, 128, 1, 128>;
        case 512: return hydro_tile_kernel<1, RECON, RIEMANN, 512, 1, 256>;
        default: return hydro_tile_kernel<1, RECON, RIEMANN, 256, 1, 256>;
    }
}

template <int RECON, int RIEMANN>
static TileKernel pick_2d(int tile)
{
    switch (tile) {
        case 1: return hydro_tile_kernel<2, RECON, RIEMANN, 32, 8, 256>;
        case 3: return hydro_tile_kernel<2, RECON, RIEMANN, 64, 8, 256>;
        case 4: return hydro_tile_kernel<2, RECON, RIEMANN, 32, 16, 256, false, true>;
        default: return hydro_tile_kernel<2, RECON, RIEMANN, 32, 16, 256>;
    }
}

static TileKernel kernel_for(const MaraBatch* b, int dim)
{
    const bool plm = b->cfg.recon == MARA_RECON_PLM, hllc = b->cfg.riemann == MARA_RIEMANN_HLLC;
    if (dim == 1) {
        if (plm) return hllc ? pick_1d<RECON_PLM, RIEMANN_HLLC>(b->tile1) : pick_1d<RECON_PLM, RIEMANN_HLLE>(b->tile1);
        return hllc ? pick_1d<RECON_PCM, RIEMANN_HLLC>(b->tile1) : pick_1d<RECON_PCM, RIEMANN_HLLE>(b->tile1);
    }
    if (plm) return hllc ? pick_2d<RECON_PLM, RIEMANN_HLLC>(b->tile2) : pick_2d<RECON_PLM, RIEMANN_HLLE>(b->tile2);
    return hllc ? pick_2d<RECON_PCM, RIEMANN_HLLC>(b->tile2) : pick_2d<RECON_PCM, RIEMANN_HLLE>(b->tile2);
}

static void tile_dims(const MaraBatch* b, int dim, int* tx, int* ty, int* nt)
{
    if (dim == 1) { *tx = b->tile1; *ty = 1; *nt = b->tile1 == 128 ? 128 : 256; return; }
    *nt = 256;
    if (b->tile2 == 1) { *tx = 32; *ty = 8; }
    else if (b->tile2 == 3) { *tx = 64; *ty = 8; }
    else { *tx = 32; *ty = 16; }
}

static int cuda_rc(cudaError_t e) { return e == cudaSuccess ? MARA_OK : MARA_ERR_CUDA; }
#define BK(call) do { const cudaError_t e_ = (call); if (e_ != cudaSuccess) return MARA_ERR_CUDA; } while (0)

static const float B_TABLE[3][3] = {{1.f, 0.f, 0.f}, {1.f, 0.5f, 0.f}, {1.f, 0.25f, 2.f / 3.f}};

static int list_mask(const MaraBatch* b) { return (b->count[0] > 0 ? 1 : 0) | (b->count[1] > 0 ? 2 : 0); }

static void enqueue_batch_step(MaraBatch* b, int mask)
{
    const int n = b->nslots, nb = (n + 255) / 256;
    const cudaStream_t s = b->stream;
    const int order = b->cfg.rk_order;
    k_batch_begin<<<nb, 256, 0, s>>>(n, b->cflbits, b->cflp, b->t, b->tfin, b->dt, b->done, b->steps, b->rot, b->pend,
                                     order == 1 ? 1 : 0);
    for (int rk = 0; rk < order; ++rk) {
        const int last = rk == order - 1;
        const float bb = B_TABLE[order - 1][rk];
        for (int d = 0; d < 2; ++d) {
            if (!(mask & (1 << d))) continue;
            int tx, ty, nt;
            tile_dims(b, d + 1, &tx, &ty, &nt);
            TileKernel k = kernel_for(b, d + 1);
            k<<<b->ctas[d], nt, 0, s>>>(b->grids, b->tiles[d], b->ntiles + d, b->rot, b->dt, 1, b->done, 1, rk, bb,
                                        1.f - bb, last, b->cflbits, 1, 0);
        }
    }
}

template <int RECON, int RIEMANN, int T1, int TY2>
static const void* persistent_fn(int mask)
{
    // a kernel serving only one of the lists needs fewer registers
    if (mask == 1) return (const void*) batch_step_kernel<RECON, RIEMANN, T1, 16, 1>;
    if (mask == 2) return (const void*) batch_step_kernel<RECON, RIEMANN, 256, TY2, 2>;
    return (const void*) batch_step_kernel<RECON, RIEMANN, T1, TY2, 3>;
}

// the persistent kernel for the batch's scheme, tile shapes and non-empty
// tile lists (mask), or null when the shapes have no persistent form (1-D
// tiles of 128 zones, 64 x 8 tiles)
static const void* persistent_kernel(const MaraBatch* b, int mask)
{
    const bool plm = b->cfg.recon == MARA_RECON_PLM, hllc = b->cfg.riemann == MARA_RIEMANN_HLLC;
    if ((b->tile1 != 256 && b->tile1 != 512) || (b->tile2 != 1 && b->tile2 != 2)) return nullptr;
    const int k = (plm ? 8 : 0) + (hllc ? 4 : 0) + (b->tile1 == 512 ? 2 : 0) + (b->tile2 == 2 ? 1 : 0);
    switch (k) {
        case 0: return persistent_fn<RECON_PCM, RIEMANN_HLLE, 256, 8>(mask);
        case 1: return persistent_fn<RECON_PCM, RIEMANN_HLLE, 256, 16>(mask);
        case 2: return persistent_fn<RECON_PCM, RIEMANN_HLLE, 512, 8>(mask);
        case 3: return persistent_fn<RECON_PCM, RIEMANN_HLLE, 512, 16>(mask);
        case 4: return persistent_fn<RECON_PCM, RIEMANN_HLLC, 256, 8>(mask);
        case 5: return persistent_fn<RECON_PCM, RIEMANN_HLLC, 256, 16>(mask);
        case 6: return persistent_fn<RECON_PCM, RIEMANN_HLLC, 512, 8>(mask);
        case 7: return persistent_fn<RECON_PCM, RIEMANN_HLLC, 512, 16>(mask);
        case 8: return persistent_fn<RECON_PLM, RIEMANN_HLLE, 256, 8>(mask);
        case 9: return persistent_fn<RECON_PLM, RIEMANN_HLLE, 256, 16>(mask);
        case 10: return persistent_fn<RECON_PLM, RIEMANN_HLLE, 512, 8>(mask);
        case 11: return persistent_fn<RECON_PLM, RIEMANN_HLLE, 512, 16>(mask);
        case 12: return persistent_fn<RECON_PLM, RIEMANN_HLLC, 256, 8>(mask);
        case 13: return persistent_fn<RECON_PLM, RIEMANN_HLLC, 256, 16>(mask);
        case 14: return persistent_fn<RECON_PLM, RIEMANN_HLLC, 512, 8>(mask);
        default: return persistent_fn<RECON_PLM, RIEMANN_HLLC, 512, 16>(mask);
    }
}

static cudaError_t launch_persistent(MaraBatch* b, int mask)
{
    BatchArgs A;
    A.grids = b->grids;
    A.tiles1 = b->tiles[0];
    A.tiles2 = b->tiles[1];
    A.ntiles = b->ntiles;
    A.rot = b->rot;
    A.t = b->t;
    A.dt = b->dt;
    A.tfin = b->tfin;
    A.cflp = b->cflp;
    A.done = b->done;
    A.pend = b->pend;
    A.steps = b->steps;
    A.cflbits = b->cflbits;
    A.bar = b->bar;
    A.err = b->kerr;
    A.nslots = b->nslots;
    A.order = b->cfg.rk_order;
    A.flip = b->cfg.rk_order == 1 ? 1 : 0;
    for (int k = 0; k < 3; ++k) A.b[k] = B_TABLE[A.order - 1][k];
    void* args[] = {(void*) &A};
    return cudaLaunchCooperativeKernel(persistent_kernel(b, mask), dim3(b->pgrid[mask]), dim3(256), args, 0,
                                       b->stream);
}

static int launches_per_step(const MaraBatch* b)
{
    const int mask = list_mask(b);
    return 1 + b->cfg.rk_order * ((mask & 1) + ((mask >> 1) & 1));
}

// one launch advancing every grid of cluster class k by nsteps steps, on
// the class's side stream
template <int RECON, int RIEMANN>
static cudaError_t launch_class(MaraBatch* b, int k, int nsteps)
{
    Cluster1DJob job = {};
    job.grids = b->grids;
    job.slots = b->cl_slots[k];
    job.t = b->t;
    job.steps = b->steps;
    job.dt = b->dt;
    job.done = b->done;
    job.cfl = b->cflbits;
    job.tfin = b->tfin;
    job.cflp = b->cflp;
    job.done_value = 2;
    job.order = b->cfg.rk_order;
    job.nsteps = nsteps;
    job.buffer = 0;   // no rotation: the clusters update in place
    return launch_cluster1d<RECON, RIEMANN>(job, b->cl_count[k], CLUSTER_BUCKET_C[k], CLUSTER_BUCKET_M[k],
                                            b->side[k]);
}

static cudaError_t launch_cluster_class(MaraBatch* b, int k, int nsteps)
{
    const bool hllc = b->cfg.riemann == MARA_RIEMANN_HLLC;
    if (b->cfg.recon == MARA_RECON_PCM)
        return hllc ? launch_class<RECON_PCM, RIEMANN_HLLC>(b, k, nsteps)
                    : launch_class<RECON_PCM, RIEMANN_HLLE>(b, k, nsteps);
    return hllc ? launch_class<RECON_PLM, RIEMANN_HLLC>(b, k, nsteps)
                : launch_class<RECON_PLM, RIEMANN_HLLE>(b, k, nsteps);
}

// steps per round of the cluster classes: about as long as the round's batch
// steps (damped: the clusters and the tile kernels share the SMs)
static void adapt_cluster_steps(MaraBatch* b)
{
    if (!b->round_open) return;
    b->round_open = false;
    float main_ms = 0.f;
    if (!b->round_mask || cudaEventElapsedTime(&main_ms, b->ev_start, b->ev_main_end) != cudaSuccess) return;
    for (int k = 0; k < CLUSTER_BUCKETS; ++k) {
        float side_ms = 0.f;
        if (!b->round_side[k] || cudaEventElapsedTime(&side_ms, b->ev_start, b->ev_side_end[k]) != cudaSuccess ||
            !(side_ms > 0.f))
            continue;
        const double f = std::sqrt((double) main_ms / side_ms);
        b->cl_steps[k] = (int) std::min(4096.0, std::max(16.0, b->cl_steps[k] * f));
    }
}

static int upload_tiles(MaraBatch* b)
{
    // rebuild both lists from the resident grids into the free pinned buffer
    const int which = b->tiles_buf ^ 1;
    BK(cudaEventSynchronize(b->tiles_ev[which]));
    int count[2] = {0, 0};
    int ccount[CLUSTER_BUCKETS] = {};
    for (int sl = 0; sl < b->nslots; ++sl) {
        const SlotHost& h = b->slots[sl];
        if (!h.used || h.finished_reported) continue;
        if (h.cluster) {
            b->cl_host[h.bucket][which][ccount[h.bucket]++] = sl;
            continue;
        }
        const int d = h.dims - 1;
        int tx, ty, nt;
        tile_dims(b, h.dims, &tx, &ty, &nt);
        for (int y = 0; y < h.n1; y += ty)
            for (int x = 0; x < h.n0; x += tx) {
                if (count[d] >= b->max_tiles[d]) return MARA_ERR_NO_ROOM;
                b->tiles_host[d][which][count[d]++] = {sl, x, y, 0};
            }
    }
    for (int d = 0; d < 2; ++d) {
        if (count[d]) BK(cudaMemcpyAsync(b->tiles[d], b->tiles_host[d][which], sizeof(TileRef) * count[d],
                                         cudaMemcpyHostToDevice, b->stream));
        k_set_int<<<1, 1, 0, b->stream>>>(b->ntiles + d, count[d]);
        b->count[d] = count[d];
    }
    for (int k = 0; k < CLUSTER_BUCKETS; ++k) {
        if (ccount[k]) BK(cudaMemcpyAsync(b->cl_slots[k], b->cl_host[k][which], sizeof(int) * ccount[k],
                                          cudaMemcpyHostToDevice, b->stream));
        b->cl_count[k] = ccount[k];
    }
    BK(cudaEventRecord(b->tiles_ev[which], b->stream));
    b->tiles_buf = which;
    b->dirty = false;
    return MARA_OK;
}

extern "C" {

int mara_batch_create(const MaraBatchConfig* c, MaraBatch** out)
{
    if (!c || !out) return MARA_ERR_ARGUMENT;
    *out = nullptr;
    if (c->max_grids < 1 || c->hbm_budget_bytes <= 0 || c->max_zones_per_grid < 1) return MARA_ERR_CONFIG;
    if (c->recon != MARA_RECON_PCM && c->recon != MARA_RECON_PLM) return MARA_ERR_CONFIG;
    if (c->rk_order < 1 || c->rk_order > 3 || c->riemann < 0 || c->riemann > 1) return MARA_ERR_CONFIG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || c->device < 0 || c->device >= ndev) return MARA_ERR_NO_DEVICE;
    BK(cudaSetDevice(c->device));
    MaraBatch* b = new (std::nothrow) MaraBatch();
    if (!b) return MARA_ERR_ARGUMENT;
    b->cfg = *c;
    b->nslots = c->max_grids;
    b->tile1 = (c->tile_1d == 128 || c->tile_1d == 256 || c->tile_1d == 512) ? c->tile_1d : 256;
    b->tile2 = (c->tile_2d >= 1 && c->tile_2d <= 4) ? c->tile_2d : 2;
    b->clusters = !c->lockstep_1d;
    for (int k = 0; k < CLUSTER_BUCKETS; ++k) b->cl_steps[k] = 256;
    b->slots.resize(b->nslots);
    b->done_host.assign(b->nslots, 1);
    int rc = MARA_OK;
    auto A = [&](void** p, size_t bytes) {
        if (rc) return;
        if (cudaMalloc(p, bytes) != cudaSuccess) rc = MARA_ERR_CUDA;
    };
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) { delete b; return MARA_ERR_CUDA; }
    cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, c->device);
    const int n = b->nslots;
    A((void**) &b->grids, sizeof(HGrid) * n);
    A((void**) &b->rot, sizeof(int) * n);
    A((void**) &b->t, sizeof(double) * n);
    A((void**) &b->dt, sizeof(double) * n);
    A((void**) &b->tfin, sizeof(double) * n);
    A((void**) &b->cflp, sizeof(double) * n);
    A((void**) &b->done, sizeof(int) * n);
    A((void**) &b->pend, sizeof(int) * n);
    A((void**) &b->steps, sizeof(long long) * n);
    A((void**) &b->cflbits, sizeof(unsigned long long) * n);
    A((void**) &b->ntiles, sizeof(int) * 2);
    A((void**) &b->bar, sizeof(unsigned) * 2);
    A((void**) &b->kerr, sizeof(int));
    // tile capacity: the budget bounds the zones resident at once
    const int64_t max_zones = c->hbm_budget_bytes / 40 + 1;   // >= 2 buffers x 20 B per zone
    b->max_tiles[0] = (int) std::min<int64_t>(max_zones / 128 + n + 16, 1 << 26);
    b->max_tiles[1] = (int) std::min<int64_t>(max_zones / 256 + 4 * n + 16, 1 << 26);
    for (int d = 0; d < 2; ++d) {
        A((void**) &b->tiles[d], sizeof(TileRef) * b->max_tiles[d]);
        for (int w = 0; w < 2 && !rc; ++w)
            if (cudaMallocHost((void**) &b->tiles_host[d][w], sizeof(TileRef) * b->max_tiles[d]) != cudaSuccess)
                rc = MARA_ERR_CUDA;
    }
    b->staging_elems = (int64_t) c->max_zones_per_grid * 5 + 1024;
    A((void**) &b->staging, sizeof(double) * b->staging_elems);
    for (int w = 0; w < 2 && !rc; ++w)
        if (cudaEventCreateWithFlags(&b->tiles_ev[w], cudaEventDisableTiming) != cudaSuccess) rc = MARA_ERR_CUDA;
    for (int k = 0; k < CLUSTER_BUCKETS && !rc; ++k) {
        A((void**) &b->cl_slots[k], sizeof(int) * n);
        for (int w = 0; w < 2 && !rc; ++w)
            if (cudaMallocHost((void**) &b->cl_host[k][w], sizeof(int) * n) != cudaSuccess) rc = MARA_ERR_CUDA;
        if (!rc && cudaStreamCreateWithFlags(&b->side[k], cudaStreamNonBlocking) != cudaSuccess) rc = MARA_ERR_CUDA;
        if (!rc && cudaEventCreate(&b->ev_side_end[k]) != cudaSuccess) rc = MARA_ERR_CUDA;
    }
    if (!rc && (cudaEventCreate(&b->ev_start) != cudaSuccess || cudaEventCreate(&b->ev_main_end) != cudaSuccess))
        rc = MARA_ERR_CUDA;
    if (!rc) {
        cudaMemsetAsync(b->done, 0, sizeof(int) * n, b->stream);
        std::vector<int> ones(n, 1);
        cudaMemcpy(b->done, ones.data(), sizeof(int) * n, cudaMemcpyHostToDevice);
        cudaMemset(b->ntiles, 0, sizeof(int) * 2);
        cudaMemset(b->bar, 0, sizeof(unsigned) * 2);
        cudaMemset(b->kerr, 0, sizeof(int));
        cudaMemset(b->rot, 0, sizeof(int) * n);
        cudaMemset(b->pend, 0, sizeof(int) * n);
        for (int d = 0; d < 2; ++d) {
            int tx, ty, nt, per = 0;
            tile_dims(b, d + 1, &tx, &ty, &nt);
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, (const void*) kernel_for(b, d + 1), nt, 0);
            b->ctas[d] = std::max(1, per) * b->sms;
        }
        // the persistent form: every CTA resident (a cooperative launch),
        // ctas_per_sm of them per SM up to what the kernel's resources allow
        int coop = 0;
        cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, c->device);
        if (c->persistent && coop && persistent_kernel(b, 3)) {
            b->persistent = true;
            for (int mask = 1; mask <= 3; ++mask) {
                int per = 0;
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, persistent_kernel(b, mask), 256, 0);
                const int want = c->ctas_per_sm > 0 ? c->ctas_per_sm : per;
                b->pgrid[mask] = std::min(want, per) * b->sms;
                if (per <= 0) b->persistent = false;
            }
        }
        rc = cuda_rc(cudaDeviceSynchronize());
    }
    if (rc) { mara_batch_destroy(b); return rc; }
    *out = b;
    return MARA_OK;
}

int mara_batch_destroy(MaraBatch* b)
{
    if (!b) return MARA_OK;
    cudaSetDevice(b->cfg.device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    for (int k = 0; k < CLUSTER_BUCKETS; ++k) {
        if (b->side[k]) { cudaStreamSynchronize(b->side[k]); cudaStreamDestroy(b->side[k]); }
        if (b->ev_side_end[k]) cudaEventDestroy(b->ev_side_end[k]);
        cudaFree(b->cl_slots[k]);
        for (int w = 0; w < 2; ++w) if (b->cl_host[k][w]) cudaFreeHost(b->cl_host[k][w]);
    }
    if (b->ev_start) cudaEventDestroy(b->ev_start);
    if (b->ev_main_end) cudaEventDestroy(b->ev_main_end);
    for (auto& g : b->graph) if (g) cudaGraphExecDestroy(g);
    cudaFree(b->bar);
    cudaFree(b->kerr);
    cudaFree(b->pend);
    for (auto& h : b->slots)
        for (int k = 0; k < 6; ++k)
            if (h.bufs[k]) cudaFree(h.bufs[k]);
    cudaFree(b->grids); cudaFree(b->rot); cudaFree(b->t); cudaFree(b->dt); cudaFree(b->tfin); cudaFree(b->cflp);
    cudaFree(b->done); cudaFree(b->steps); cudaFree(b->cflbits); cudaFree(b->ntiles); cudaFree(b->staging);
    for (int d = 0; d < 2; ++d) {
        cudaFree(b->tiles[d]);
        for (int w = 0; w < 2; ++w) if (b->tiles_host[d][w]) cudaFreeHost(b->tiles_host[d][w]);
    }
    for (int w = 0; w < 2; ++w) if (b->tiles_ev[w]) cudaEventDestroy(b->tiles_ev[w]);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return MARA_OK;
}

int mara_batch_admit(MaraBatch* b, const MaraGpuConfig* c, const double* P_aos, double t_final, double cfl, int* slot)
{
    if (!b || !c || !P_aos) return MARA_ERR_ARGUMENT;
    if (c->law != MARA_LAW_HYDRO || c->nk != 1 || c->ni < 2) return MARA_ERR_CONFIG;
    if (c->recon != b->cfg.recon || c->riemann != b->cfg.riemann || c->rk_order != b->cfg.rk_order) return MARA_ERR_CONFIG;
    const int s_need = c->recon == MARA_RECON_PCM ? 1 : 2;
    const int dims = c->nj > 1 ? 2 : 1;
    if (c->ng[0] < s_need || (dims == 2 && c->ng[1] < s_need)) return MARA_ERR_GUARD_TOO_SMALL;
    const int64_t zones = (int64_t) c->ni * c->nj;
    const int N0 = c->ni + 2 * c->ng[0], N1 = c->nj + 2 * (dims == 2 ? c->ng[1] : 0);
    if ((int64_t) N0 * N1 * 5 > b->staging_elems) return MARA_ERR_TOO_LARGE;
    const int nbuf = b->cfg.rk_order == 3 ? 3 : 2;
    const int64_t bytes = (int64_t) nbuf * 2 * 5 * zones * 4;
    int sl = -1;
    for (int k = 0; k < b->nslots; ++k)
        if (!b->slots[k].used) { sl = k; break; }
    if (sl < 0 || b->bytes_in_use + bytes > b->cfg.hbm_budget_bytes) return MARA_ERR_NO_ROOM;
    BK(cudaSetDevice(b->cfg.device));
    SlotHost& h = b->slots[sl];
    h = SlotHost();
    for (int k = 0; k < 2 * nbuf; ++k) {
        if (cudaMallocAsync((void**) &h.bufs[k], sizeof(float) * 5 * zones, b->stream) != cudaSuccess) {
            for (int j = 0; j < k; ++j) cudaFreeAsync(h.bufs[j], b->stream);
            return MARA_ERR_NO_ROOM;
        }
    }
    h.used = true;
    h.dims = dims;
    h.n0 = c->ni;
    h.n1 = c->nj;
    h.g0 = c->ng[0];
    h.g1 = dims == 2 ? c->ng[1] : 0;
    h.bc = c->bc;
    h.gamma = c->gamma;
    h.bytes = bytes;
    h.zones = zones;
    h.cluster = b->clusters && dims == 1 && c->ni <= CLUSTER_MAX_ZONES && t_final >= 0.0;
    h.bucket = h.cluster ? cluster_bucket(c->ni) : 0;
    b->bytes_in_use += bytes;

    HGrid g;
    std::memset(&g, 0, sizeof(g));
    for (int k = 0; k < nbuf; ++k) { g.Uh[k] = h.bufs[2 * k]; g.Ul[k] = h.bufs[2 * k + 1]; }
    g.sU = zones;
    g.n0 = c->ni;
    g.n1 = c->nj;
    g.bc = c->bc;
    g.gamma = (float) c->gamma;
    g.plm_theta = (float) c->plm_theta;
    const double dx = (c->upper[0] - c->lower[0]) / c->ni, dy = (c->upper[1] - c->lower[1]) / c->nj;
    const double dz = (c->upper[2] - c->lower[2]) / c->nk;
    g.idx = (float) (1.0 / dx);
    g.idy = (float) (1.0 / dy);
    g.lmin = (float) std::min(dx, std::min(dy, dz));

    BK(cudaMemcpyAsync(b->staging, P_aos, sizeof(double) * (size_t) N0 * N1 * 5, cudaMemcpyHostToDevice, b->stream));
    k_slot_init<<<1, 1, 0, b->stream>>>(b->grids, b->rot, b->t, b->dt, b->tfin, b->cflp, b->done, b->steps, b->pend,
                                        sl, g, t_final, cfl, h.cluster ? CLUSTER_RUNNING : 0);
    k_set_u64<<<1, 1, 0, b->stream>>>(b->cflbits + sl, ~0ull);
    dim3 grid((c->ni + 255) / 256, c->nj);
    k_batch_load<<<grid, 256, 0, b->stream>>>(b->staging, g, h.g0, h.g1, N0, N1, 1.0 / (c->gamma - 1.0),
                                              b->cflbits + sl);
    b->launches += 3;
    b->done_host[sl] = 0;
    b->dirty = true;
    *slot = sl;
    return cuda_rc(cudaGetLastError());
}

int mara_batch_step(MaraBatch* b, int steps)
{
    if (!b) return MARA_ERR_ARGUMENT;
    BK(cudaSetDevice(b->cfg.device));
    if (b->dirty) {
        const int rc = upload_tiles(b);
        if (rc) return rc;
        b->launches += 2;
    }
    const int mask = list_mask(b);
    if (!b->persistent && !b->graph[mask]) {
        cudaGraph_t g;
        BK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        enqueue_batch_step(b, mask);
        BK(cudaStreamEndCapture(b->stream, &g));
        const cudaError_t e = cudaGraphInstantiate(&b->graph[mask], g, 0);
        cudaGraphDestroy(g);
        BK(e);
    }
    // the cluster classes first, so that their CTAs are placed while the
    // batch steps queue behind them on the main stream
    bool side = false;
    for (int k = 0; k < CLUSTER_BUCKETS; ++k) side = side || b->cl_count[k] > 0;
    if (side && steps > 0) {
        BK(cudaEventRecord(b->ev_start, b->stream));
        for (int k = 0; k < CLUSTER_BUCKETS; ++k) {
            b->round_side[k] = b->cl_count[k] > 0;
            if (!b->round_side[k]) continue;
            BK(cudaStreamWaitEvent(b->side[k], b->ev_start, 0));
            BK(launch_cluster_class(b, k, mask ? b->cl_steps[k] : 1024));
            BK(cudaEventRecord(b->ev_side_end[k], b->side[k]));
            b->launches += 1;
        }
    }
    if (b->persistent && steps > 0) {
        if (mask) {
            for (int k = 0; k < steps; ++k) BK(launch_persistent(b, mask));
            b->launches += steps;
        }
    } else {
        for (int k = 0; k < steps; ++k) BK(cudaGraphLaunch(b->graph[mask], b->stream));
        b->launches += (int64_t) steps * launches_per_step(b);
    }
    if (side && steps > 0) {
        BK(cudaEventRecord(b->ev_main_end, b->stream));
        for (int k = 0; k < CLUSTER_BUCKETS; ++k)
            if (b->round_side[k]) BK(cudaStreamWaitEvent(b->stream, b->ev_side_end[k], 0));
        b->round_open = true;
        b->round_mask = mask;
    }
    b->step_count += steps;
    return MARA_OK;
}

int mara_batch_poll(MaraBatch* b, int* slots, int cap, int* n)
{
    if (!b || !n) return MARA_ERR_ARGUMENT;
    BK(cudaSetDevice(b->cfg.device));
    std::vector<int> d(b->nslots);
    BK(cudaMemcpyAsync(d.data(), b->done, sizeof(int) * b->nslots, cudaMemcpyDeviceToHost, b->stream));
    BK(cudaStreamSynchronize(b->stream));
    if (b->persistent) {
        int err = 0;
        BK(cudaMemcpy(&err, b->kerr, sizeof(int), cudaMemcpyDeviceToHost));
        if (err) return MARA_ERR_CUDA;   // a barrier wait gave up: the batch's state is not usable
    }
    adapt_cluster_steps(b);
    int m = 0;
    for (int k = 0; k < b->nslots; ++k) {
        SlotHost& h = b->slots[k];
        if (h.used && !h.finished_reported && d[k] == 2) {
            h.finished_reported = true;
            b->dirty = true;  // its tiles leave the lists
            if (m < cap && slots) slots[m] = k;
            ++m;
        }
    }
    *n = m;
    return MARA_OK;
}

int mara_batch_retire(MaraBatch* b, int slot, double* P_aos, double* t, int64_t* steps)
{
    if (!b || slot < 0 || slot >= b->nslots || !b->slots[slot].used) return MARA_ERR_ARGUMENT;
    BK(cudaSetDevice(b->cfg.device));
    SlotHost& h = b->slots[slot];
    const int N0 = h.n0 + 2 * h.g0, N1 = h.n1 + 2 * h.g1;
    HGrid g;
    std::memset(&g, 0, sizeof(g));
    BK(cudaMemcpyAsync(&g, b->grids + slot, sizeof(HGrid), cudaMemcpyDeviceToHost, b->stream));
    int rot = 0;
    double tt = 0;
    long long st = 0;
    BK(cudaMemcpyAsync(&rot, b->rot + slot, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
    BK(cudaMemcpyAsync(&tt, b->t + slot, sizeof(double), cudaMemcpyDeviceToHost, b->stream));
    BK(cudaMemcpyAsync(&st, b->steps + slot, sizeof(long long), cudaMemcpyDeviceToHost, b->stream));
    BK(cudaStreamSynchronize(b->stream));
    if (P_aos) {
        const long long cells = (long long) N0 * N1;
        k_batch_store<<<(unsigned) ((cells + 255) / 256), 256, 0, b->stream>>>(g, rot, h.g0, h.g1, N0, N1, h.gamma,
                                                                              b->staging);
        BK(cudaMemcpyAsync(P_aos, b->staging, sizeof(double) * cells * 5, cudaMemcpyDeviceToHost, b->stream));
        b->launches += 1;
    }
    k_slot_clear<<<1, 1, 0, b->stream>>>(b->done, slot);
    for (int k = 0; k < 6; ++k)
        if (h.bufs[k]) cudaFreeAsync(h.bufs[k], b->stream);
    BK(cudaStreamSynchronize(b->stream));
    b->bytes_in_use -= h.bytes;
    b->zone_updates += h.zones * st;
    if (t) *t = tt;
    if (steps) *steps = st;
    b->done_host[slot] = 1;
    h = SlotHost();
    b->dirty = true;
    return MARA_OK;
}

int mara_batch_stats(MaraBatch* b, MaraBatchStats* s)
{
    if (!b || !s) return MARA_ERR_ARGUMENT;
    std::memset(s, 0, sizeof(*s));
    for (const auto& h : b->slots) {
        if (!h.used) continue;
        if (h.finished_reported) s->finished++;
        else { s->active++; s->zones += h.zones; }
    }
    s->bytes_in_use = b->bytes_in_use;
    s->zone_updates = b->zone_updates;
    s->steps = b->step_count;
    s->kernel_launches = b->launches;
    return MARA_OK;
}

int mara_batch_tiles(MaraBatch* b, int* t1, int* t2)
{
    if (!b) return MARA_ERR_ARGUMENT;
    if (t1) *t1 = b->tile1;
    if (t2) *t2 = b->tile2;
    return MARA_OK;
}

} // extern "C"

int mara_batch_launch_form(MaraBatch* b, int* persistent, int* ctas)
{
    if (!b || !persistent || !ctas) return MARA_ERR_ARGUMENT;
    *persistent = b->persistent ? 1 : 0;
    *ctas = b->persistent ? b->pgrid[3] : b->ctas[1];
    return MARA_OK;
}
