// gw_engine.cuh -- the cluster-resident multi-step engine kernel and its launcher.
// Included by gw_kernel_fp64.cu and gw_kernel_fp32.cu, which instantiate one precision each.
#pragma once

#include <type_traits>

#include "gw_kernel.cuh"

namespace gw {
namespace dev {

// Per-warp flux partial, 32 bytes in both precisions:
//   FP32: {JLCC hi, lo, Jxfer hi, lo, Jtr hi, lo, ClCh count, 0} (float pairs, TwoSum-compensated)
//   FP64: {JLCC, Jxfer, Jtr, ClCh count}
struct Partial {
    double v[4];
};

struct OdeShared {
    double g[kNumGlobals];
    double sv[kSvCount];
    double expm;
    double t;
    double sums[4];  // JLCC, ClCh, Jtr, Jxfer
    int status;
    int pad;
};

struct SmemLayout {
    size_t cc, sv, ode, part, tile, total;
};

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

template <typename R>
__host__ __device__ inline SmemLayout smem_layout(int ssa_warps, int tile_cap, int max_cta_cell) {
    SmemLayout L;
    size_t o = 0;
    L.cc = o;
    o += align16(sizeof(SsaConsts<R>));
    L.sv = o;
    o += align16(2 * kSvCount * sizeof(R));
    L.ode = o;
    o += align16(sizeof(OdeShared));
    L.part = o;
    o += align16((size_t)2 * max_cta_cell * ssa_warps * sizeof(Partial));
    L.tile = o;
    // lcc, flags, ryr[6] (u32), cass[4], jlcc[4], cajsr (R), cajsr_lo (f32)
    o += align16((size_t)tile_cap * (8 * sizeof(uint32_t) + 9 * sizeof(R) + sizeof(float)));
    L.total = o;
    return L;
}

// double-float accumulate: (hi, lo) += (bh, bl)
__device__ __forceinline__ void df_add(float &hi, float &lo, float bh, float bl) {
    const float s = hi + bh;
    const float bb = s - hi;
    float e = (hi - (s - bb)) + (bh - bb);
    e += lo + bl;
    hi = s + e;
    lo = e - (hi - s);
}

__device__ __forceinline__ bool finite_bits(double x) {
    return ((__double_as_longlong(x) >> 52) & 0x7FF) != 0x7FF;
}

// Stimulus of step ri at time t (pulse train or per-step samples).  Uses explicit round-to-nearest
// operations so the host's evaluation of the same pulse train gives the same values.
__device__ __forceinline__ double stimulus(const CellDyn &d, double t, int64_t ri) {
    if (d.stim_mode == STIM_SAMPLES) return (ri >= 0 && ri < d.stim_n) ? d.stim_samples[ri] : 0.0;
    if (d.stim_mode == STIM_PULSE) {
        double tb = __dsub_rn(t, d.stim_start);
        if (tb >= 0.0) {
            if (d.stim_period > 0.0)
                tb = __dsub_rn(tb, __dmul_rn(d.stim_period, trunc(__ddiv_rn(tb, d.stim_period))));
            if (tb < d.stim_dur) return d.stim_amp;
        }
    }
    return 0.0;
}

template <bool FP64>
__device__ __forceinline__ void push_sv(const OdeShared &os, void *svbuf, int slot,
                                        const CtaWork &w, int lane) {
    using R = typename std::conditional<FP64, double, float>::type;
    R *sv = reinterpret_cast<R *>(svbuf) + slot * kSvCount;
    for (int i = lane; i < kSvCount; i += 32) {
        R v = (R)os.sv[i];
        if (!FP64) {
            if (i == SV_CAI_LO) v = (R)(os.sv[SV_CAI] - (double)(float)os.sv[SV_CAI]);
            if (i == SV_CANSR_LO) v = (R)(os.sv[SV_CANSR] - (double)(float)os.sv[SV_CANSR]);
        }
        for (int r = 0; r < w.n_cta_cell; ++r) st_remote(map_rank(sv + i, (uint32_t)(w.first + r)), v);
    }
}

// Lane-parallel reduction of the cell's per-warp partials of one slot; lane 0 returns the sums
// {JLCC, ClCh, Jtr, Jxfer} in FP64.
template <bool FP64>
__device__ __forceinline__ void reduce_partials(const Partial *slot, int n, int lane, double *out) {
    if (FP64) {
        double a = 0, b = 0, c = 0, d = 0;
        for (int i = lane; i < n; i += 32) {
            a += slot[i].v[0];
            b += slot[i].v[1];
            c += slot[i].v[2];
            d += slot[i].v[3];
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_xor_sync(0xffffffffu, a, o);
            b += __shfl_xor_sync(0xffffffffu, b, o);
            c += __shfl_xor_sync(0xffffffffu, c, o);
            d += __shfl_xor_sync(0xffffffffu, d, o);
        }
        if (lane == 0) {
            out[0] = a;  // JLCC
            out[1] = d;  // ClCh
            out[2] = c;  // Jtr
            out[3] = b;  // Jxfer
        }
    } else {
        float jh = 0, jl = 0, xh = 0, xl = 0, th = 0, tl = 0;
        int cl = 0;
        for (int i = lane; i < n; i += 32) {
            const float *f = reinterpret_cast<const float *>(slot[i].v);
            df_add(jh, jl, f[0], f[1]);
            df_add(xh, xl, f[2], f[3]);
            df_add(th, tl, f[4], f[5]);
            cl += (int)f[6];
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float a0 = __shfl_xor_sync(0xffffffffu, jh, o), a1 = __shfl_xor_sync(0xffffffffu, jl, o);
            const float b0 = __shfl_xor_sync(0xffffffffu, xh, o), b1 = __shfl_xor_sync(0xffffffffu, xl, o);
            const float c0 = __shfl_xor_sync(0xffffffffu, th, o), c1 = __shfl_xor_sync(0xffffffffu, tl, o);
            cl += __shfl_xor_sync(0xffffffffu, cl, o);
            df_add(jh, jl, a0, a1);
            df_add(xh, xl, b0, b1);
            df_add(th, tl, c0, c1);
        }
        if (lane == 0) {
            out[0] = (double)jh + (double)jl;
            out[1] = (double)cl;
            out[2] = (double)th + (double)tl;
            out[3] = (double)xh + (double)xl;
        }
    }
}

constexpr int kMaxThreads = 512;  // SSA warps + ODE warp per CTA (128 registers per thread)

template <bool FP64, bool ODE64>
__global__ void __launch_bounds__(kMaxThreads, 1) engine_kernel(const KernelArgs a) {
    using R = typename std::conditional<FP64, double, float>::type;
    using T = typename std::conditional<ODE64, double, float>::type;
    constexpr bool EXACT = FP64;
    extern __shared__ __align__(16) unsigned char smem[];
    const int nw = a.ssa_warps;
    const int warp = (int)(threadIdx.x >> 5), lane = (int)(threadIdx.x & 31);
    const CtaWork w = a.work[blockIdx.x];
    const bool active = w.cell >= 0;
    const bool leader = active && w.rank_in_cell == 0;
    const SmemLayout L = smem_layout<R>(nw, a.tile_cap, a.max_cta_cell);
    SsaConsts<R> &cc = *reinterpret_cast<SsaConsts<R> *>(smem + L.cc);
    R *svbuf = reinterpret_cast<R *>(smem + L.sv);
    OdeShared &os = *reinterpret_cast<OdeShared *>(smem + L.ode);
    Partial *part = reinterpret_cast<Partial *>(smem + L.part);
    const int cap = a.tile_cap;
    uint32_t *t_lcc = reinterpret_cast<uint32_t *>(smem + L.tile);
    uint32_t *t_flags = t_lcc + cap;
    uint32_t *t_ryr = t_flags + cap;
    R *t_cass = reinterpret_cast<R *>(t_ryr + 6 * cap);
    R *t_jlcc = t_cass + 4 * cap;
    R *t_cajsr = t_jlcc + 4 * cap;
    float *t_cajsr_lo = reinterpret_cast<float *>(t_cajsr + cap);
    const int cell = w.cell;
    const int pslot = a.max_cta_cell * nw;  // partial entries per parity slot
    R *g_cass = reinterpret_cast<R *>(a.cass);
    R *g_jlcc = reinterpret_cast<R *>(a.jlcc);
    R *g_cajsr = reinterpret_cast<R *>(a.cajsr);

    uint64_t step0 = 0;
    if (active) {
        if (threadIdx.x == 0) load_ssa_consts<R>(cc, a.cs[cell]);
        step0 = a.dyn[cell].step;
        if (warp < nw) {
            const int64_t base = a.slot0[cell] + w.cru_begin;
            for (int m = (int)threadIdx.x; m < w.cru_count; m += nw * 32) {
                const int64_t gs = base + m;
                t_lcc[m] = a.lcc[gs];
                t_flags[m] = a.flags[gs];
#pragma unroll
                for (int k = 0; k < 6; ++k) t_ryr[k * cap + m] = a.ryr[k * a.n_slots + gs];
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    t_cass[j * cap + m] = g_cass[j * a.n_slots + gs];
                    t_jlcc[j * cap + m] = g_jlcc[j * a.n_slots + gs];
                }
                t_cajsr[m] = g_cajsr[gs];
                if (!FP64) t_cajsr_lo[m] = a.cajsr_lo[gs];
            }
        }
    }
    if (leader && warp == nw) {
        if (lane == 0) {
            const CellDyn &d = a.dyn[cell];
            for (int i = 0; i < kNumGlobals; ++i) os.g[i] = d.g[i];
            os.t = d.t;
            os.sums[0] = d.sum_jlcc;
            os.sums[1] = d.sum_clch;
            os.sums[2] = d.sum_jtr;
            os.sums[3] = d.sum_jxfer;
            os.status = 0;
            os.expm = step_values(a.cs[cell], os.g, os.sv);
        }
        __syncwarp();
        push_sv<FP64>(os, svbuf, 0, w, lane);
    }
    __syncthreads();
    cluster_sync();

    const R dt = (R)a.dt;
    unsigned long long my_events = 0;
    int my_err = 0;
    for (int s = 0; s < a.n_steps; ++s) {
        const int par = s & 1;
        const int64_t ri = a.run_step0 + s;
        const bool rec = a.record_every > 0 && (ri % a.record_every) == 0;
        const int64_t r_idx = rec ? ri / a.record_every - a.rec_base : -1;
        const bool rec_ok = rec && r_idx >= 0 && r_idx < a.rec_cap;
        if (warp < nw) {
            if (active) {
                const R *sv = svbuf + par * kSvCount;
                float jh = 0, jl = 0, xh = 0, xl = 0, th = 0, tl = 0;
                double dj = 0, dx = 0, dtr = 0;
                int acl = 0;
                for (int m = (int)threadIdx.x; m < w.cru_count; m += nw * 32) {
                    Cru<R> c;
                    c.lcc = t_lcc[m];
                    c.flags = t_flags[m];
#pragma unroll
                    for (int k = 0; k < 6; ++k) c.ryr[k] = t_ryr[k * cap + m];
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        c.cass[j] = t_cass[j * cap + m];
                        c.jlcc[j] = t_jlcc[j * cap + m];
                    }
                    c.cajsr = t_cajsr[m];
                    c.cajsr_lo = FP64 ? 0.f : t_cajsr_lo[m];
                    Stream rng;
                    rng.open(a.seed, (uint32_t)cell, (uint32_t)(w.cru_begin + m), step0 + s, 0);
                    R jx, jt;
                    int ev = 0, err = 0;
                    ssa_cru<R, EXACT>(c, cc, sv, rng, dt, a.event_cap, jx, jt, ev, err);
                    t_lcc[m] = c.lcc;
                    t_flags[m] = c.flags;
#pragma unroll
                    for (int k = 0; k < 6; ++k) t_ryr[k * cap + m] = c.ryr[k];
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        t_cass[j * cap + m] = c.cass[j];
                        t_jlcc[j * cap + m] = c.jlcc[j];
                    }
                    t_cajsr[m] = c.cajsr;
                    if (!FP64) t_cajsr_lo[m] = c.cajsr_lo;
                    my_events += (unsigned long long)ev;
                    my_err |= err;
                    const R jsum = c.jlcc[0] + c.jlcc[1] + c.jlcc[2] + c.jlcc[3];
                    if (FP64) {
                        dj += (double)jsum;
                        dx += (double)jx;
                        dtr += (double)jt;
                    } else {
                        df_add(jh, jl, (float)jsum, 0.f);
                        df_add(xh, xl, (float)jx, 0.f);
                        df_add(th, tl, (float)jt, 0.f);
                    }
                    acl += __popc((c.flags >> 4) & 0xFu);
                    if (rec_ok && cell == a.tr_cell) {
                        const int64_t cm = w.cru_begin + m;
                        const int64_t st = a.tr_cru_stride;
                        a.tr_lcc[r_idx * st + cm] = c.lcc;
                        a.tr_flags[r_idx * st + cm] = c.flags;
#pragma unroll
                        for (int k = 0; k < 6; ++k) a.tr_ryr[(r_idx * 6 + k) * st + cm] = c.ryr[k];
#pragma unroll
                        for (int j = 0; j < 4; ++j)
                            reinterpret_cast<R *>(a.tr_cass)[(r_idx * 4 + j) * st + cm] = c.cass[j];
                        reinterpret_cast<R *>(a.tr_cajsr)[r_idx * st + cm] = c.cajsr;
                    }
                }
                // warp reduction and push of the partial to the leader CTA
                Partial pv;
                if (FP64) {
                    double dcl = (double)acl;
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) {
                        dj += __shfl_xor_sync(0xffffffffu, dj, o);
                        dx += __shfl_xor_sync(0xffffffffu, dx, o);
                        dtr += __shfl_xor_sync(0xffffffffu, dtr, o);
                        dcl += __shfl_xor_sync(0xffffffffu, dcl, o);
                    }
                    pv.v[0] = dj;
                    pv.v[1] = dx;
                    pv.v[2] = dtr;
                    pv.v[3] = dcl;
                } else {
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) {
                        const float a0 = __shfl_xor_sync(0xffffffffu, jh, o), a1 = __shfl_xor_sync(0xffffffffu, jl, o);
                        const float b0 = __shfl_xor_sync(0xffffffffu, xh, o), b1 = __shfl_xor_sync(0xffffffffu, xl, o);
                        const float c0 = __shfl_xor_sync(0xffffffffu, th, o), c1 = __shfl_xor_sync(0xffffffffu, tl, o);
                        acl += __shfl_xor_sync(0xffffffffu, acl, o);
                        df_add(jh, jl, a0, a1);
                        df_add(xh, xl, b0, b1);
                        df_add(th, tl, c0, c1);
                    }
                    float *f = reinterpret_cast<float *>(pv.v);
                    f[0] = jh; f[1] = jl; f[2] = xh; f[3] = xl; f[4] = th; f[5] = tl;
                    f[6] = (float)acl;
                    f[7] = 0.f;
                }
                if (lane < 4) {
                    Partial *dst = part + par * pslot + w.rank_in_cell * nw + warp;
                    const double v = lane == 0 ? pv.v[0] : lane == 1 ? pv.v[1] : lane == 2 ? pv.v[2] : pv.v[3];
                    st_remote(map_rank(&dst->v[lane], (uint32_t)w.first), v);
                }
            }
        } else if (leader) {
            // The cell's global step s -> s+1 with the fluxes of step s-1, concurrently with the
            // SSA warps' step s.
            double sums[4];
            if (s > 0) reduce_partials<FP64>(part + (par ^ 1) * pslot, w.n_cta_cell * nw, lane, sums);
            if (lane == 0) {
                if (s == 0) {
                    sums[0] = os.sums[0];
                    sums[1] = os.sums[1];
                    sums[2] = os.sums[2];
                    sums[3] = os.sums[3];
                }
                const CellStatic &C = a.cs[cell];
                const double Istim = stimulus(a.dyn[cell], os.t, ri);
                int st = ode_step<T>(C, os.g, sums, Istim, a.dt, os.expm);
                os.t += a.dt;
                bool fin = true;
                for (int i = 0; i < kNumGlobals; ++i) fin = fin && finite_bits(os.g[i]);
                if (!fin && st == 0) st = GW_ERR_NONFINITE;
                if (st != 0 && os.status == 0) os.status = st;
                if (rec_ok) {
                    double *dst = a.tr_glob + ((int64_t)cell * a.rec_cap + r_idx) * kNumGlobals;
                    for (int i = 0; i < kNumGlobals; ++i) dst[i] = os.g[i];
                    if (cell == 0 || (a.tr_cell >= 0 && cell == a.tr_cell)) a.tr_t[r_idx] = os.t;
                }
                os.expm = step_values(C, os.g, os.sv);
            }
            __syncwarp();
            push_sv<FP64>(os, svbuf, par ^ 1, w, lane);
        }
        cluster_sync();
    }

    // Epilogue: carry of the last step's fluxes, globals and counters back to the cell block.
    if (leader && warp == nw) {
        double sums[4];
        if (a.n_steps > 0)
            reduce_partials<FP64>(part + ((a.n_steps - 1) & 1) * pslot, w.n_cta_cell * nw, lane, sums);
        if (lane == 0) {
            CellDyn &d = a.dyn[cell];
            if (a.n_steps > 0) {
                d.sum_jlcc = sums[0];
                d.sum_clch = sums[1];
                d.sum_jtr = sums[2];
                d.sum_jxfer = sums[3];
            }
            for (int i = 0; i < kNumGlobals; ++i) d.g[i] = os.g[i];
            d.t = os.t;
            d.step = step0 + (uint64_t)a.n_steps;
            if (os.status != 0) atomicCAS(&a.status[cell], 0, os.status);
        }
    }
    if (active && warp < nw) {
        const int64_t base = a.slot0[cell] + w.cru_begin;
        for (int m = (int)threadIdx.x; m < w.cru_count; m += nw * 32) {
            const int64_t gs = base + m;
            a.lcc[gs] = t_lcc[m];
            a.flags[gs] = t_flags[m];
#pragma unroll
            for (int k = 0; k < 6; ++k) a.ryr[k * a.n_slots + gs] = t_ryr[k * cap + m];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                g_cass[j * a.n_slots + gs] = t_cass[j * cap + m];
                g_jlcc[j * a.n_slots + gs] = t_jlcc[j * cap + m];
            }
            g_cajsr[gs] = t_cajsr[m];
            if (!FP64) a.cajsr_lo[gs] = t_cajsr_lo[m];
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            my_events += __shfl_xor_sync(0xffffffffu, my_events, o);
            my_err |= __shfl_xor_sync(0xffffffffu, my_err, o);
        }
        if (lane == 0) {
            if (my_events) atomicAdd(a.events, my_events);
            if (my_err) atomicCAS(&a.status[cell], 0, (int)GW_ERR_EVENT_CAP);
        }
    }
}

// Random initial CRU state (GW_utils.tpp:5-64) from stream 1, one thread per CRU, in the same
// draw order as the oracle's orc_sample_initial_crus.
template <bool FP64>
__global__ void init_crus_kernel(const KernelArgs a, int cell, int ncru) {
    using R = typename std::conditional<FP64, double, float>::type;
    const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (i >= ncru) return;
    Stream s;
    s.open(a.seed, (uint32_t)cell, (uint32_t)i, 0, 1);
    uint32_t k = 0;
    auto pick = [&](const double *w, int n) {
        const double u = FP64 ? s.u53(k) : (double)s.u24(k);
        ++k;
        const double uu = u * 1.0;
        double cum = w[0];
        int idx = 0;
        while (cum < uu && idx < n - 1) {
            ++idx;
            cum += w[idx];
        }
        return idx;
    };
    const double wl[3] = {0.958, 0.038, 0.004};
    const double wi[2] = {0.9425, 0.0575};
    const double wr[3] = {0.609, 0.5 * 0.391, 0.5 * 0.391};
    const double wc[2] = {0.998, 0.002};
    const int lcc_of[3] = {1, 2, 7};
    const int ryr_of[3] = {0, 4, 5};
    uint32_t lcc = 0, flags = 0, ryr[6] = {0, 0, 0, 0, 0, 0};
    for (int j = 0; j < 4; ++j) lcc = byte_set(lcc, j, lcc_of[pick(wl, 3)]);
    for (int j = 0; j < 4; ++j)
        if (pick(wi, 2) == 0) flags |= (1u << j);
    for (int j = 0; j < 4; ++j)
        for (int q = 0; q < 5; ++q) {
            const int st = ryr_of[pick(wr, 3)];
#pragma unroll
            for (int z = 0; z < 6; ++z)
                if (z == st) ryr[z] = byte_add(ryr[z], j, 1);
        }
    for (int j = 0; j < 4; ++j)
        if (pick(wc, 2) == 1) flags |= (1u << (4 + j));
    const int64_t gs = a.slot0[cell] + i;
    a.lcc[gs] = lcc;
    a.flags[gs] = flags;
    for (int z = 0; z < 6; ++z) a.ryr[z * a.n_slots + gs] = ryr[z];
    R *cass = reinterpret_cast<R *>(a.cass);
    R *jlcc = reinterpret_cast<R *>(a.jlcc);
    for (int j = 0; j < 4; ++j) {
        cass[j * a.n_slots + gs] = (R)1.45370e-4;
        jlcc[j * a.n_slots + gs] = (R)0;
    }
    reinterpret_cast<R *>(a.cajsr)[gs] = (R)0.908408;
    if (!FP64) a.cajsr_lo[gs] = (float)(0.908408 - (double)(float)0.908408);
}

template <bool FP64>
inline int launch_engine(const KernelArgs &a, const LaunchShape &s, void *stream, bool ode64) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)s.ctas, 1, 1);
    cfg.blockDim = dim3((unsigned)s.threads, 1, 1);
    cfg.dynamicSmemBytes = s.smem;
    cfg.stream = (cudaStream_t)stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)s.cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaError_t e;
    if (ode64) {
        auto k = engine_kernel<FP64, true>;
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s.smem);
        cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        e = cudaLaunchKernelEx(&cfg, k, a);
    } else {
        auto k = engine_kernel<FP64, false>;
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s.smem);
        cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        e = cudaLaunchKernelEx(&cfg, k, a);
    }
    return (int)e;
}

template <bool FP64>
inline int max_active_clusters(const LaunchShape &s, bool ode64, int *out) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)s.ctas, 1, 1);
    cfg.blockDim = dim3((unsigned)s.threads, 1, 1);
    cfg.dynamicSmemBytes = s.smem;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)s.cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaError_t e;
    if (ode64) {
        auto k = engine_kernel<FP64, true>;
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s.smem);
        cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        e = cudaOccupancyMaxActiveClusters(out, k, &cfg);
    } else {
        auto k = engine_kernel<FP64, false>;
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s.smem);
        cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        e = cudaOccupancyMaxActiveClusters(out, k, &cfg);
    }
    return (int)e;
}

}  // namespace dev
}  // namespace gw
