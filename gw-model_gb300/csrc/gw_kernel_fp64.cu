// FP64 engine (reference semantics).  Compiled with -fmad=false so that products and sums round
// as the reference's separate multiply and add do.
#include "gw_engine.cuh"

namespace gw {

int launch_engine_fp64(const KernelArgs &a, const LaunchShape &s, void *stream, bool ode64) {
    return dev::launch_engine<true>(a, s, stream, ode64);
}
size_t smem_bytes_fp64(int tile_cap, int max_cta_cell) {
    return dev::smem_layout<double, double>(tile_cap, max_cta_cell).total;
}
int max_active_clusters_fp64(const LaunchShape &s, bool ode64, int *out) {
    return dev::max_active_clusters<true>(s, ode64, out);
}
int sample_initial_crus_dev(const KernelArgs &a, int cell, int ncru, int fp64, void *stream) {
    const int threads = 256;
    const int blocks = (ncru + threads - 1) / threads;
    if (fp64)
        dev::init_crus_kernel<true><<<blocks, threads, 0, (cudaStream_t)stream>>>(a, cell, ncru);
    else
        dev::init_crus_kernel<false><<<blocks, threads, 0, (cudaStream_t)stream>>>(a, cell, ncru);
    return (int)cudaGetLastError();
}

namespace dev {
// The global step's FP64 exp and log (gw_math64.cuh) on n inputs, for their accuracy check.
__global__ void math_check_kernel(const double *x, int n, double *ex, double *lg) {
    __shared__ math64::Tables T;
    math64::load_tables(T, (int)threadIdx.x, (int)blockDim.x);
    __syncthreads();
    const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (i >= n) return;
    ex[i] = math64::exp(x[i], T);
    lg[i] = math64::log(x[i], T);
}
}  // namespace dev

int math_check_dev(const double *x, int n, double *ex, double *lg) {
    if (n <= 0) return 0;
    const int threads = 256;
    dev::math_check_kernel<<<(n + threads - 1) / threads, threads>>>(x, n, ex, lg);
    return (int)cudaGetLastError();
}

}  // namespace gw
