// no_alloc.cu -- mara_gpu_advance_noalloc: one plain-FP64 MethodOfLinesTVD
// advance on caller-owned device buffers, with every intermediate array
// (primitive ping-pong buffers, stage conserved states, face fluxes, status)
// carved out of a fixed scratch array that is part of this library's device
// image.  Nothing here allocates: no cudaMalloc, cudaFree, cudaMallocAsync or
// allocating library call.
//
// Who needs this: callers that cannot allocate device memory when they step
// a grid -- a host application whose own memory pool has already reserved
// the GPU's memory, a latency-critical loop that must not block in (or fail
// inside) an allocation halfway through a run, or code that must not trigger
// the implicit device-wide synchronisation of cudaFree.
//
// Limits and sharing rules:
//   * the scratch array holds MARA_NOALLOC_SCRATCH_BYTES (64 MiB) on every
//     GPU that loads the library, for as long as the process runs; a grid
//     whose intermediates do not fit is rejected with MARA_ERR_TOO_LARGE;
//   * every call uses the same array and leaves its contents behind; the
//     status words are cleared at the start of each call, everything else is
//     fully overwritten before it is read;
//   * calls whose GPU work overlaps (on different streams, or from different
//     threads) race on the array: order them on one stream;
//   * every call looks up the array's device address (cudaGetSymbolAddress,
//     host-side, allocates nothing) with config->device current, so a
//     context that was torn down and created again is followed; the first
//     call on a device may load the library's device image there, so make
//     it before any stream capture;
//   * the caller's current device is restored before the call returns.
#include <cuda_runtime.h>

#include <cstring>

#include "../../include/mara_gpu.h"
#include "internal.h"

#define MARA_NOALLOC_SCRATCH_BYTES (64ull << 20)

// The scratch array.  In host code its name is only a host-side stand-in:
// kernels must be given the device address looked up below.
static __device__ __align__(256) unsigned char mara_noalloc_scratch[MARA_NOALLOC_SCRATCH_BYTES];

namespace mara {

// declared here, defined in mara_gpu.cu: configuration checks and mesh
// description shared with the handle-based entry points
int noalloc_validate(const MaraGpuConfig* c);
void noalloc_make_grid(const MaraGpuConfig* c, GridDesc* G);

__global__ void k_noalloc_begin(DevStatus* st, double dt)
{
    DevStatus z;
    memset(&z, 0, sizeof(z));
    z.first_zone = ~0ull;
    z.dt = dt;
    *st = z;
}

static size_t round_up(size_t n) { return (n + 255) & ~size_t(255); }

// the advance proper, with config->device current
static int noalloc_advance(const MaraGpuConfig* config, const GridDesc& G, size_t pbytes, size_t ubytes,
                           size_t fbytes, const double* P_in, double* P_out, double dt, cudaStream_t s)
{
    // the scratch array's device address in the current context
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, mara_noalloc_scratch) != cudaSuccess || !p) return MARA_ERR_CUDA;
    unsigned char* cur = (unsigned char*) p;

    // carve the scratch array
    DevStatus* st = (DevStatus*) cur;
    cur += round_up(sizeof(DevStatus));
    double* P[2];
    P[0] = (double*) cur; cur += pbytes;
    P[1] = (double*) cur; cur += pbytes;
    double* U0 = (double*) cur; cur += ubytes;
    double* U = (double*) cur; cur += ubytes;
    double* F[3] = {nullptr, nullptr, nullptr};
    for (int a = 0; a < 3; ++a)
        if (G.n[a] > 1) { F[a] = (double*) cur; cur += fbytes; }

    PhysParamsH pp;
    make_phys(config, &pp);
    const int law = kernel_law(config);

    // status cleared and dt set; the AoS input is fully transposed into P[0]
    k_noalloc_begin<<<1, 1, 0, s>>>(st, dt);
    launch_aos_to_soa(P_in, P[0], G, s);

    // the RK stages of MethodOfLinesTVD::advance (SolutionSchemes.cpp:191-274)
    static const double b1[1] = {1.0};
    static const double b2[2] = {1.0, 0.5};
    static const double b3[3] = {1.0, 1. / 4, 2. / 3};
    const double* b = config->rk_order == 1 ? b1 : config->rk_order == 2 ? b2 : b3;
    int c = 0;
    for (int rk = 0; rk < config->rk_order; ++rk) {
        for (int a = 0; a < 3; ++a)
            if (G.n[a] > 1) plain_flux(law, config->recon, config->riemann, a, G, pp, P[c], F[a], st, s);
        plain_update(law, G, pp, P[c], P[1 - c], U0, U, F[0], F[1], F[2], b[rk], rk, &st->dt, st, s);
        c = 1 - c;
    }
    launch_soa_to_aos(P[c], P_out, G, s);
    // launch errors of this call only: checked before anything else runs
    if (cudaGetLastError() != cudaSuccess) return MARA_ERR_CUDA;

    DevStatus host;
    if (cudaMemcpyAsync(&host, st, sizeof(DevStatus), cudaMemcpyDeviceToHost, s) != cudaSuccess) return MARA_ERR_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return MARA_ERR_CUDA;
    if (host.code) return host.code;
    if (host.failures > 0) return MARA_ERR_INVERSION_FAILURE;
    return MARA_OK;
}

} // namespace mara

using namespace mara;

extern "C" int mara_gpu_advance_noalloc(const MaraGpuConfig* config, const double* P_in, double* P_out,
                                        double dt, void* stream)
{
    if (!config || !P_in || !P_out) return MARA_ERR_ARGUMENT;
    const int v = noalloc_validate(config);
    if (v) return v;
    if (config->precision != MARA_PRECISION_FP64) return MARA_ERR_CONFIG;

    GridDesc G;
    noalloc_make_grid(config, &G);
    const size_t pbytes = round_up(sizeof(double) * (size_t) G.sP * G.nq);
    const size_t ubytes = round_up(sizeof(double) * (size_t) G.sU * G.nq);
    const size_t fbytes = round_up(sizeof(double) * (size_t) G.sF * G.nq);
    int axes = 0;
    for (int a = 0; a < 3; ++a) axes += G.n[a] > 1;
    const size_t need = round_up(sizeof(DevStatus)) + 2 * pbytes + 2 * ubytes + axes * fbytes;
    if (need > MARA_NOALLOC_SCRATCH_BYTES) return MARA_ERR_TOO_LARGE;

    int prev = -1;
    if (cudaGetDevice(&prev) != cudaSuccess) return MARA_ERR_NO_DEVICE;
    if (prev != config->device && cudaSetDevice(config->device) != cudaSuccess) return MARA_ERR_NO_DEVICE;
    const int rc = noalloc_advance(config, G, pbytes, ubytes, fbytes, P_in, P_out, dt, (cudaStream_t) stream);
    if (prev != config->device) cudaSetDevice(prev);
    return rc;
}
