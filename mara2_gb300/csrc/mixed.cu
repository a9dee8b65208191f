// mixed.cu -- placeholder until the mixed-precision kernels land.
#include "mixed.h"

namespace mara {
struct MixedState { int parity; };
int mixed_create(const MaraGpuConfig*, const GridDesc&, MixedState** out, cudaStream_t, int64_t*) { *out = nullptr; return MARA_ERR_CONFIG; }
void mixed_destroy(MixedState*) {}
void mixed_load_aos(MixedState*, const double*, cudaStream_t) {}
void mixed_store_aos(MixedState*, double*, cudaStream_t) {}
void mixed_enqueue_step(MixedState*, const double*, DevStatus*, cudaStream_t, int64_t*) {}
void mixed_enqueue_courant(MixedState*, DevStatus*, cudaStream_t) {}
int mixed_launches_per_step(const MixedState*) { return 0; }
int mixed_parity(const MixedState* m) { return m->parity; }
void mixed_set_parity(MixedState* m, int p) { m->parity = p; }
void mixed_advance_parity(MixedState*) {}
void mixed_set_timing(MixedState*, int) {}
void mixed_kernel_times(MixedState*, double*, int64_t*) {}
}
