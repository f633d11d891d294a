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
// The FP64 lane's FP32 screen (SsaLane::surely_last) beside the FP64 iteration's own decision, for
// n given CRU states, step values, times and step lengths (draw 0 of stream (seed, cell 0, CRU i,
// step 0)): out[2i] the screen's verdict, out[2i+1] whether the FP64 iteration was the step's last,
// jump[i] its jump time when it was not.
__global__ void screen_check_kernel(const CellStatic *cs, int n, const uint32_t *chan, const double *cass,
                                    const double *sv, const double *t, const double *dt, uint64_t seed, int *out,
                                    double *jump) {
    __shared__ SsaConsts<double> cc;
    __shared__ float sk[SK_COUNT];
    if (threadIdx.x == 0) {
        load_ssa_consts<double>(cc, *cs);
        load_screen_consts(sk, *cs);
    }
    __syncthreads();
    const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (i >= n) return;
    Cru<double> c;
    c.lcc = chan[8 * (int64_t)i];
    c.flags = chan[8 * (int64_t)i + 1];
    for (int q = 0; q < 6; ++q) c.ryr[q] = chan[8 * (int64_t)i + 2 + q];
    for (int j = 0; j < 4; ++j) {
        c.cass[j] = cass[4 * (int64_t)i + j];
        c.jlcc[j] = 0.0;
    }
    c.cajsr = 1.0;
    c.cajsr_lo = 0.f;
    const double *svi = sv + (int64_t)kSvCount * i;
    float svf[kSvCount];
    for (int e = 0; e < kSvCount; ++e) svf[e] = (float)svi[e];
    Stream rng;
    rng.open(seed, 0u, (uint32_t)i, 0ull, 0u);
    SsaLane<double, true> L;
    L.begin(c, cc);
    L.t = t[i];
    const bool sc = L.surely_last(c, cc, sk, svf, rng, dt[i]);
    IterInfo<double> f;
    int err = 0;
    L.iterate(c, cc, svi, nullptr, rng, dt[i], 1 << 30, err, &f);
    out[2 * (int64_t)i] = sc ? 1 : 0;
    out[2 * (int64_t)i + 1] = f.act == 0 ? 1 : 0;
    jump[i] = f.act == 0 ? 0.0 : f.h;
}
}  // namespace dev

int screen_check_dev(const CellStatic *cs, int n, const uint32_t *chan, const double *cass, const double *sv,
                     const double *t, const double *dt, uint64_t seed, int *out, double *jump) {
    if (n <= 0) return 0;
    const int threads = 128;
    dev::screen_check_kernel<<<(n + threads - 1) / threads, threads>>>(cs, n, chan, cass, sv, t, dt, seed, out, jump);
    return (int)cudaGetLastError();
}

int math_check_dev(const double *x, int n, double *ex, double *lg) {
    if (n <= 0) return 0;
    const int threads = 256;
    dev::math_check_kernel<<<(n + threads - 1) / threads, threads>>>(x, n, ex, lg);
    return (int)cudaGetLastError();
}

}  // namespace gw
