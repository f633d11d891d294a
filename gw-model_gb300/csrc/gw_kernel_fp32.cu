// FP32 engine (FP32 CRU state and propensities; FP64 global state).
#include "gw_engine.cuh"

namespace gw {

int launch_engine_fp32(const KernelArgs &a, const LaunchShape &s, void *stream, bool ode64) {
    return dev::launch_engine<false>(a, s, stream, ode64);
}
size_t smem_bytes_fp32(int tile_cap, int max_cta_cell) {
    return dev::smem_layout<float, double>(tile_cap, max_cta_cell).total;
}
int max_active_clusters_fp32(const LaunchShape &s, bool ode64, int *out) {
    return dev::max_active_clusters<false>(s, ode64, out);
}

}  // namespace gw
