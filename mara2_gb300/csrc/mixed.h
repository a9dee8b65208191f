// mixed.h -- the mixed-precision path's interface to the C ABI layer.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/mara_gpu.h"
#include "internal.h"

namespace mara {

struct MixedState;

int mixed_create(const MaraGpuConfig* c, const GridDesc& G, MixedState** out, cudaStream_t s, int64_t* bytes);
void mixed_destroy(MixedState* m);
// upload: begin, then the AoS cells [c0, c1) as their copies land, then finish
void mixed_load_begin(MixedState* m, cudaStream_t s);
void mixed_load_aos_range(MixedState* m, const double* aos, long long c0, long long c1, DevStatus* st, cudaStream_t s);
void mixed_load_finish(MixedState* m, DevStatus* st, cudaStream_t s);
void mixed_store_aos_range(MixedState* m, double* aos, long long c0, long long c1, cudaStream_t s);
void mixed_enqueue_step(MixedState* m, const double* dt, DevStatus* st, cudaStream_t s, int64_t* timed);
void mixed_enqueue_courant(MixedState* m, DevStatus* st, cudaStream_t s);
// One whole driver-loop step (dt from the Courant step, stages, clock) or one
// advance with a given dt, when the fused hydro kernels apply; false (nothing
// enqueued) otherwise.
bool mixed_enqueue_run_step(MixedState* m, double cfl, double t_final, DevStatus* st, cudaStream_t s);
bool mixed_enqueue_advance(MixedState* m, double dt, DevStatus* st, cudaStream_t s);
void mixed_sync_rotation(MixedState* m, cudaStream_t s);
// one advance of a page-locked host MeshData::P in place (host_dev: its
// device address), the transfers and the stages pipelined in one launch
// (2-D fused grids)
// MIXED_NOT_TAKEN: the pipelined step cannot run on this device (it then
// stays off for the handle); nothing was changed, use the unpipelined path
constexpr int MIXED_NOT_TAKEN = -1;
bool mixed_host_step_capable(const MixedState* m);
int mixed_advance_host_step(MixedState* m, double* host_dev, double dt, DevStatus* st, cudaStream_t s,
                            int64_t* launches);
int mixed_launches_per_step(const MixedState* m);
bool mixed_fused(const MixedState* m);
// 1-D hydro grids of up to 8192 zones on the fused form: up to nsteps
// driver-loop steps in one launch on a thread-block cluster holding the grid
// in shared memory (hydro_cluster.cuh)
bool mixed_cluster_capable(const MixedState* m);
int mixed_enqueue_cluster_steps(MixedState* m, int nsteps, double cfl, double t_final, DevStatus* st, cudaStream_t s);
int mixed_parity(const MixedState* m);
void mixed_set_parity(MixedState* m, int p);
void mixed_advance_parity(MixedState* m);
void mixed_set_timing(MixedState* m, int on);
void mixed_kernel_times(MixedState* m, double ms[3], int64_t launches[3]);
// FP32 primitives with guards of the general form (nullptr for the fused form)
const float* mixed_primitives(const MixedState* m);
// volume-integrated diagnostics of the state a download would return
// (partial: DIAG_BLOCKS x 17 doubles; err: first error code; out: totals)
void mixed_volume_diagnostics(MixedState* m, double* partial, int* err, double* out, cudaStream_t s);

} // namespace mara
