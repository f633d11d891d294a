// gw_engine.cuh -- the cluster-resident multi-step engine kernel and its launcher.
// Included by gw_kernel_fp64.cu and gw_kernel_fp32.cu, which instantiate one precision each.
//
// CTA = ssa_warps + kOdeWarps warps.  In a cell's leader CTA the last kOdeWarps warps run the
// global step as the lane program of gw_ode_program.h; in the other CTAs of the cell every warp
// runs SSA.  The CTAs of a cell are held together only by their data, which travel by st.async
// and complete per-parity mbarriers of the receiver (no cluster barrier inside the launch):
//   SSA warps : wait for sv[s&1] (the CTA's mbarrier), then each warp runs the SSA of step s on a
//               contiguous range of the CTA's CRU tile, one CRU per lane at a time; a lane whose
//               CRU has finished its step takes the warp's next CRU, so lanes with pending SSA
//               events do not hold the others back.  Each warp pushes its flux partial into its
//               slot in the leader's shared memory.
//   ODE warps : wait for the warp partials of step s-1 (the leader's mbarrier), reduce them,
//               increments and Euler update (globals s -> s+1), transcendental phases of the new
//               state (an idle lane forms the stimulus of step s+1), push sv[(s+1)&1]; phases the
//               SSA does not need run after the push.
#pragma once

#include <type_traits>

#include "gw_kernel.cuh"
#include "gw_math64.cuh"
#include "gw_ode_program.h"

namespace gw {
namespace dev {

// Flux partial of a warp or a CTA, 32 bytes in both precisions:
//   FP32: {JLCC hi, lo, Jxfer hi, lo, Jtr hi, lo, ClCh count, 0} (float pairs, TwoSum-compensated)
//   FP64: {JLCC, Jxfer, Jtr, ClCh count}
struct Partial {
    double v[4];
};

struct OdeShared {
    double g[kNumGlobals];  // the cell's globals (FP64 state)
    double t;               // accumulated time
    double sums[4];         // JLCC, ClCh, Jtr, Jxfer sums of the last reduced step (FP64)
    double stim[2];         // stimulus of step s in slot s & 1, from the leader's SSA warps
    int status;
    int pad;
};

constexpr int kMaxThreads = 512;  // SSA warps + ODE warps per CTA (128 registers per thread)
constexpr int kMaxThreadsFp64 = 256;  // FP64 instance: at most 4 SSA warps, up to 255 registers
constexpr int kMaxWarps = kMaxThreads / 32;

struct SmemLayout {
    size_t cc, sv, ode, prog, x, math, svs, rtab, part, mbar, fq, tile, total;
};

// FP64: CRUs of a CTA whose first iteration of a step waits for the four-lane pass (the queue
// holds their tile indices; a CTA with more such CRUs in a step runs the rest on their own lanes).
constexpr int kEngQCap = 256;

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

template <typename R, typename T>
__host__ __device__ inline SmemLayout smem_layout(int tile_cap, int max_cta_cell) {
    SmemLayout L;
    size_t o = 0;
    L.cc = o;
    o += align16(sizeof(SsaConsts<R>));
    L.sv = o;
    o += align16(2 * kSvCount * sizeof(R));
    L.ode = o;
    o += align16(sizeof(OdeShared));
    L.prog = o;
    o += align16(sizeof(OdeProgram));
    L.x = o;
    o += align16(kOdeMaxSlots * sizeof(T));
    L.math = o;  // exp / log tables of the FP64 global step
    o += align16(sizeof(math64::Tables));
    L.svs = o;   // staging of the per-step SSA values before the push
    o += align16(kSvCount * sizeof(R));
    L.rtab = o;  // the CTA's subunit rate tables (FP32 SSA), one per step parity
    o += align16((size_t)2 * kRateTab * sizeof(float2));
    L.part = o;  // [parity][rank in cell][warp]: warp partials (written by the cell's CTAs)
    o += align16((size_t)2 * max_cta_cell * kMaxWarps * sizeof(Partial));
    L.mbar = o;  // mbarriers: the warp partials of steps of parity 0 and 1 (leader CTA), then the
    o += 32;     // per-step SSA values of parity 0 and 1 (every CTA)
    L.fq = o;    // FP64: the queue's two counters (by step parity), then kEngQCap tile indices
    o += sizeof(R) == 8 ? align16((size_t)(4 + kEngQCap) * sizeof(int)) : 0;
    L.tile = o;  // TileRec<R> per CRU
    o += align16((size_t)tile_cap * sizeof(TileRec<R>));
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

__device__ __forceinline__ void cluster_arrive() {
    asm volatile("barrier.cluster.arrive.release;" ::: "memory");
}
__device__ __forceinline__ void cluster_arrive_relaxed() {
    asm volatile("barrier.cluster.arrive.relaxed;" ::: "memory");
}
__device__ __forceinline__ void cluster_wait() {
    asm volatile("barrier.cluster.wait.acquire;" ::: "memory");
}
// barrier of the ODE warps (named barrier 1, kOdeLanes threads)
__device__ __forceinline__ void ode_bar() { asm volatile("bar.sync 1, %0;" ::"n"(kOdeLanes) : "memory"); }
// barrier of a CTA's SSA warps (named barrier 2, n threads: the CTA's SSA threads 0 .. n-1)
__device__ __forceinline__ void ssa_bar(int n) { asm volatile("bar.sync 2, %0;" ::"r"(n) : "memory"); }
// named barrier `id` of n threads that also returns the OR of v over them: a decision that every
// participating thread takes the same way (a bounded wait's outcome, which is per thread)
__device__ __forceinline__ bool bar_or(int id, int n, bool v) {
    int r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.s32 p, %1, 0;\n\t"
        "bar.red.or.pred q, %2, %3, p;\n\t"
        "selp.s32 %0, 1, 0, q;\n\t}"
        : "=r"(r)
        : "r"((int)v), "r"(id), "r"(n)
        : "memory");
    return r != 0;
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

// Branch of the gate rates (common.hpp:176-218): 0 for V >= -40, 2 for V == -47.13, 1 otherwise
// (NaN included), from integer compares on the bit pattern (no FP64 issue slots).
__device__ __forceinline__ int v_regime(double V) {
    const long long b = __double_as_longlong(V);
    if (b >= 0) return (unsigned long long)b > 0x7FF0000000000000ull ? 1 : 0;  // +NaN: 1
    const unsigned long long u = (unsigned long long)b;
    if (u <= 0xC044000000000000ull) return 0;  // -40 <= V <= -0
    return u == 0xC04790A3D70A3D71ull ? 2 : 1;  // V == -47.13
}

// !(x > 0) for a concentration, from the bit pattern (non-positive or NaN).
__device__ __forceinline__ bool not_positive(double x) {
    const long long b = __double_as_longlong(x);
    return b <= 0 || (unsigned long long)b > 0x7FF0000000000000ull;
}

__device__ __forceinline__ double o_exp(double x, const math64::Tables &M) { return math64::exp(x, M); }
__device__ __forceinline__ float o_exp(float x, const math64::Tables &) { return expf(x); }
__device__ __forceinline__ double o_log(double x, const math64::Tables &M) { return math64::log(x, M); }
__device__ __forceinline__ float o_log(float x, const math64::Tables &) { return logf(x); }

__device__ __forceinline__ double t_sqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float t_sqrt(float x) { return sqrtf(x); }

// Shared-memory offsets of the global step's data, passed to ode_phase in place of pointers: the
// function is out of line, and pointer arguments would turn every operand, program and table
// read into a generic load; addresses formed from the shared-memory symbol inside the function
// stay shared-memory loads.
struct OdeOffsets {
    uint32_t prog, x, ode, math, stage;
};

// The FP32 pair (hi, lo) of an FP64 value for the SSA: hi = (float)d, lo = (float)(d - hi); for an
// FP64 SSA the value itself and 0.
__device__ __forceinline__ void stage_pair(float *st, int ihi, int ilo, double d) {
    const float hi = (float)d;
    st[ihi] = hi;
    st[ilo] = (float)(d - (double)hi);
}
__device__ __forceinline__ void stage_pair(double *st, int ihi, int ilo, double d) {
    st[ihi] = d;
    st[ilo] = 0.0;
}

// One phase of the lane program by the kOdeLanes ODE threads (t = 0 .. kOdeLanes-1): thread t runs
// op t of the phase.  Every warp holds one op kind per phase (P.wkind), so the switch does not
// diverge; lanes without an op skip the arithmetic.  Kept out of line: inlined into the engine
// kernel's loop, its shuffle tree measured 4x slower (2.2k vs 0.5k cycles per SUM phase).
// An op whose output is a per-step SSA value also writes it, in the SSA's precision, to the push
// staging row (P.sv_stage); Cai and CaNSR are staged by the caller (ode_warps).
template <typename T, typename R>
__device__ __noinline__ void ode_phase(const OdeOffsets o, int q, int regime, int t) {
    extern __shared__ __align__(16) unsigned char smem[];
    R *stage = reinterpret_cast<R *>(smem + o.stage);
    const OdeProgram &P = *reinterpret_cast<const OdeProgram *>(smem + o.prog);
    T *X = reinterpret_cast<T *>(smem + o.x);
    OdeShared &os = *reinterpret_cast<OdeShared *>(smem + o.ode);
    double *g = os.g;
    const math64::Tables &M = *reinterpret_cast<const math64::Tables *>(smem + o.math);
    const int wk = P.wkind[q][t >> 5];
    if (wk == OK_NOP) return;
    const int lane = t & 31;
    const int b0 = P.phase_begin[q];
    const bool live = t < P.phase_begin[q + 1] - b0;
    const OdeOp *op = &P.ops[b0 + (live ? t : 0)];
    if (live && regime > 0) {
        const int ai = P.alt_idx[b0 + t];
        if (ai != 255) op = &P.alt[regime - 1][ai];
    }
    // the 32-byte op in two 16-byte loads: consecutive lanes read consecutive ops, so the loads do
    // not conflict on shared-memory banks (field-by-field loads at a 32-byte stride would)
    const uint4 w0 = reinterpret_cast<const uint4 *>(op)[0], w1 = reinterpret_cast<const uint4 *>(op)[1];
    const int kind = live ? (int)(w0.x & 0xFFu) : (int)OK_NOP;
    const int out = (int)(w0.x >> 16);
    const uint32_t pw[7] = {w0.y, w0.z, w0.w, w1.x, w1.y, w1.z, w1.w};
#define GW_ARG(k) (X[(pw[(k) >> 1] >> (16 * ((k) & 1))) & 0xFFFFu])
    T v = (T)0;
    if (kind != OK_NOP) {
        switch (wk) {
        case OK_LOG: v = o_log(GW_ARG(0) + GW_ARG(1) * GW_ARG(2), M); break;
        case OK_SQRT: v = GW_ARG(0) * GW_ARG(1) * t_sqrt(GW_ARG(2) * GW_ARG(3)); break;
        case OK_EXP: v = GW_ARG(0) * o_exp(GW_ARG(1) * GW_ARG(2) + GW_ARG(3), M); break;
        case OK_AFF: v = GW_ARG(0) * GW_ARG(1) + GW_ARG(2) * GW_ARG(3) + GW_ARG(4) * GW_ARG(5) + GW_ARG(6); break;
        case OK_REC:
            v = (T)1 / (GW_ARG(0) + GW_ARG(1) * GW_ARG(2) + GW_ARG(3) * GW_ARG(4) + GW_ARG(5) * GW_ARG(6) * GW_ARG(7));
            break;
        case OK_PROD: v = GW_ARG(0) * GW_ARG(1) * GW_ARG(2) * GW_ARG(3) * GW_ARG(4) * GW_ARG(5) * GW_ARG(6); break;
        case OK_SUM:
        case OK_SUMU:
            v = GW_ARG(2) * GW_ARG(3) * GW_ARG(4) + GW_ARG(5) * GW_ARG(6) * GW_ARG(7) + GW_ARG(8) * GW_ARG(9) * GW_ARG(10) +
                GW_ARG(11) * GW_ARG(12) * GW_ARG(13);
            break;
        default: break;
        }
    }
    if (wk == OK_SUM || wk == OK_SUMU) {
        // rows of `width` lanes (a power of two, rows aligned to it): tree over offsets 1, 2, 4
        const bool row = kind == OK_SUM || kind == OK_SUMU;
        const int wm = row ? (int)((w0.x >> 8) & 0xFFu) - 1 : 0;
#pragma unroll
        for (int off = 1; off < 8; off <<= 1) {
            const T o = __shfl_down_sync(0xffffffffu, v, off);
            if (row && (lane & wm) + off <= wm && (lane & (2 * off - 1)) == 0) v += o;
        }
        if (row && (lane & wm) == 0) {
            const T r = GW_ARG(0) * GW_ARG(1) * v;
            if (kind == OK_SUMU) {
                // Euler update of global `out` (FP64 state); every row of the phase reads the old
                // values at XS_G, the new one goes to XS_GN for the phases that follow
                const double ng = g[out] + (double)r;
                g[out] = ng;
                X[XS_GN + out] = (T)ng;
                if (!finite_bits(ng)) atomicCAS(&os.status, 0, (int)GW_ERR_NONFINITE);  // first error of the cell
            } else {
                X[out] = r;
                const int sv = P.sv_stage[b0 + t];
                if (sv) stage[sv - 1] = (R)r;
            }
        }
        return;
    }
#undef GW_ARG
    if (kind != OK_NOP) {
        X[out] = v;
        const int sv = P.sv_stage[b0 + t];
        if (sv) stage[sv - 1] = (R)v;
    }
}

// Sums {JLCC, ClCh, Jtr, Jxfer} of the cell's CTA partials of one slot; ODE warp w reduces
// quantity w.  Writes the FP64 sums to out[] (shared) from lane 0 of each warp.  A lane takes the
// slots lane, lane + 32, ... (at most kSlotsPerLane): all its loads are issued first and summed in
// a pairwise tree, so the lane's part costs one load latency and three dependent additions.
constexpr int kSlotsPerLane = 16 * kMaxWarps / 32;  // up to 16 CTAs per cell
template <bool FP64, typename T>
__device__ __forceinline__ void reduce_partials(const Partial *slot, int n, int warp, int lane, double *out, T *X) {
    if (warp >= 4) return;
    double r;
    if (FP64) {
        const int src = warp == 0 ? 0 : (warp == 1 ? 3 : (warp == 2 ? 2 : 1));  // JLCC, ClCh, Jtr, Jxfer
        double a[kSlotsPerLane];
#pragma unroll
        for (int k = 0; k < kSlotsPerLane; ++k) {
            const int i = lane + 32 * k;
            a[k] = i < n ? slot[i].v[src] : 0.0;
        }
#pragma unroll
        for (int w = kSlotsPerLane / 2; w > 0; w >>= 1)
#pragma unroll
            for (int k = 0; k < w; ++k) a[k] += a[k + w];
        double acc = a[0];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        r = acc;
    } else {
        // float fields: 0,1 JLCC; 2,3 Jxfer; 4,5 Jtr; 6 ClCh
        const int src = warp == 0 ? 0 : (warp == 1 ? 6 : (warp == 2 ? 4 : 2));
        float h[kSlotsPerLane], l[kSlotsPerLane];
#pragma unroll
        for (int k = 0; k < kSlotsPerLane; ++k) {
            const int i = lane + 32 * k;
            const float *f = reinterpret_cast<const float *>(slot[i < n ? i : 0].v);
            h[k] = i < n ? f[src] : 0.f;
            l[k] = i < n && warp != 1 ? f[src + 1] : 0.f;
        }
#pragma unroll
        for (int w = kSlotsPerLane / 2; w > 0; w >>= 1)
#pragma unroll
            for (int k = 0; k < w; ++k) df_add(h[k], l[k], h[k + w], l[k + w]);
        float hi = h[0], lo = l[0];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float a0 = __shfl_xor_sync(0xffffffffu, hi, o), a1 = __shfl_xor_sync(0xffffffffu, lo, o);
            df_add(hi, lo, a0, a1);
        }
        r = (double)hi + (double)lo;
    }
    if (lane == 0) {
        out[warp] = r;
        X[XS_SUMS + warp] = (T)r;
    }
}

// Per-step SSA values of the new state to every CTA of the cell: the staging row (written by the
// ops that produce the values, see ode_phase, and visible after the phase's barrier) pushed in
// 16-byte words (CTA, word) by all kOdeLanes threads, as asynchronous stores that count themselves
// off the receiving CTA's mbarrier of this slot (local shared address mbar_slot in every CTA).
template <bool FP64>
__device__ __forceinline__ void push_sv(void *svbuf, const void *stage, int slot, uint32_t mbar_slot, const CtaWork &w,
                                        int t) {
    using R = typename std::conditional<FP64, double, float>::type;
    constexpr int kWords = kSvCount * (int)sizeof(R) / 16;  // 16-byte words of one slot
    static_assert(kSvCount * sizeof(R) % 16 == 0, "sv slot in 16-byte words");
    const uint4 *src = reinterpret_cast<const uint4 *>(stage);
    uint4 *dst = reinterpret_cast<uint4 *>(reinterpret_cast<R *>(svbuf) + slot * kSvCount);
    const int total = kWords * w.n_cta_cell;
    for (int idx = t; idx < total; idx += kOdeLanes) {
        const int r = idx / kWords, i = idx - r * kWords;
        const uint32_t rank = (uint32_t)(w.first + r);
        st_async(map_rank(dst + i, rank), src[i], map_rank_addr(mbar_slot, rank));
    }
}

// Ca in 2^-40 mM fixed point (exact, order-independent sums of the record-time CRU sums).
__device__ __forceinline__ long long fix40(float x) { return __float2ll_rn(x * 0x1p40f); }
__device__ __forceinline__ long long fix40(double x) { return __double2ll_rn(x * 0x1p40); }

// The RyR states of subunit j as the int16 code of the reference's reduced-memory trace
// (utils.py:8-22): a negative count in a lumped pair (3/4, 5/6) moves the pair's total into the
// pair's first state; code = n1 + 6 n2 + 36 n3 + 216 n4 + 1296 n5.
__device__ __forceinline__ uint32_t ryr_code16(const uint32_t (&ry)[6], int j) {
    const int r0 = byte_s(ry[0], j), r1 = byte_s(ry[1], j), r2 = byte_s(ry[2], j);
    const int r3 = byte_s(ry[3], j), r4 = byte_s(ry[4], j), r5 = byte_s(ry[5], j);
    const bool n34 = r2 < 0 || r3 < 0, n56 = r4 < 0 || r5 < 0;
    const int q2 = n34 ? r2 + r3 : r2, q3 = n34 ? 0 : r3, q4 = n56 ? r4 + r5 : r4;
    return (uint32_t)(uint16_t)(int16_t)(r0 + 6 * r1 + 36 * q2 + 216 * q3 + 1296 * q4);
}

// Record step, by one warp over its CRUs [beg, end) of the tile after the step's SSA: the trace
// cell's CRU records (planes or the reduced-memory codec) and every cell's CRU sums (warp sums
// added to the record's int64 counters; integer adds, so the totals do not depend on order).
template <typename R>
__device__ __forceinline__ void record_pass(const KernelArgs &a, const CtaWork &w, int cell, int64_t r_idx, int beg,
                                            int end, int lane, const TileRec<R> *tile) {
    constexpr bool FP64 = sizeof(R) == 8;
    const bool crus = cell == a.tr_cell;
    const bool sums = a.tr_sums != nullptr;
    long long v[kSumFields] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int m = beg + lane; m < end; m += 32) {
        Cru<R> c;
        tile_get(c, tile[m]);
        const uint32_t lcc = c.lcc, fl = c.flags;
        const uint32_t(&ry)[6] = c.ryr;
        const R(&cs)[4] = c.cass;
        const R jsr = c.cajsr;
        if (sums) {
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int st = byte_u(lcc, j);
                const bool open = st == 6 || st == 12;
                const bool cond = open && ((fl >> j) & 1u);
                const long long f = fix40(cs[j]);
                v[0] += open;
                v[1] += cond;
                v[2] += cond ? f : 0;
                v[3] += byte_s(ry[2], j) + byte_s(ry[3], j);
                v[5] += f;
            }
            v[4] += __popc((fl >> 4) & 0xFu);
            v[6] += fix40(jsr) + (FP64 ? 0ll : fix40(c.cajsr_lo));
            v[7] += 1;
        }
        if (crus) {
            const int64_t cm = w.cru_begin + m;
            if (a.tr_mode == 0) {
                const int64_t st = a.tr_cru_stride;
                a.tr_lcc[r_idx * st + cm] = lcc;
                a.tr_flags[r_idx * st + cm] = fl;
#pragma unroll
                for (int k = 0; k < 6; ++k) a.tr_ryr[(r_idx * 6 + k) * st + cm] = ry[k];
#pragma unroll
                for (int j = 0; j < 4; ++j) reinterpret_cast<R *>(a.tr_cass)[(r_idx * 4 + j) * st + cm] = cs[j];
                reinterpret_cast<R *>(a.tr_cajsr)[r_idx * st + cm] = jsr;
            } else {
                const int64_t o = r_idx * a.tr_ncru + cm;
                a.tr_lcc[o] = lcc;
                a.tr_gate[o] = ((fl & 0xFu) * 0x00204081u) & 0x01010101u;
                a.tr_clch[o] = (((fl >> 4) & 0xFu) * 0x00204081u) & 0x01010101u;
                a.tr_ryrc[2 * o] = ryr_code16(ry, 0) | (ryr_code16(ry, 1) << 16);
                a.tr_ryrc[2 * o + 1] = ryr_code16(ry, 2) | (ryr_code16(ry, 3) << 16);
                reinterpret_cast<float4 *>(a.tr_cass_f)[o] =
                    make_float4((float)cs[0], (float)cs[1], (float)cs[2], (float)cs[3]);
                a.tr_cajsr_f[o] = (float)jsr;  // FP32: the compensated value rounds to its leading part
            }
        }
    }
    if (sums) {
#pragma unroll
        for (int f = 0; f < kSumFields; ++f) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v[f] += __shfl_xor_sync(0xffffffffu, v[f], o);
        }
        if (lane == 0) {
            unsigned long long *dst = a.tr_sums + ((int64_t)cell * a.rec_cap + r_idx) * kSumFields;
#pragma unroll
            for (int f = 0; f < kSumFields; ++f)
                if (v[f] != 0) atomicAdd(dst + f, (unsigned long long)v[f]);
        }
    }
}


// Per-lane flux accumulators and their warp sum as a Partial (all lanes hold it).
template <bool FP64>
struct FluxAcc {
    float jh = 0, jl = 0, xh = 0, xl = 0, th = 0, tl = 0;  // FP32: (hi, lo) pairs
    double dj = 0, dx = 0, dtr = 0;                       // FP64
    int acl = 0;
    // FP32: a lane's own CRUs (one to a few per step) add up in FP32, the lane sums in a plain
    // FP32 tree (warp_total); the cell's warp partials are then combined with compensation
    // (reduce_partials).
    __device__ __forceinline__ void add(float j, float x, float t, int cl) {
        jh += j;
        xh += x;
        th += t;
        acl += cl;
    }
    __device__ __forceinline__ void add(double j, double x, double t, int cl) {
        dj += j;
        dx += x;
        dtr += t;
        acl += cl;
    }
    __device__ __forceinline__ Partial warp_total() {
        Partial pv;
        if (FP64) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                dj += __shfl_xor_sync(0xffffffffu, dj, o);
                dx += __shfl_xor_sync(0xffffffffu, dx, o);
                dtr += __shfl_xor_sync(0xffffffffu, dtr, o);
                acl += __shfl_xor_sync(0xffffffffu, acl, o);
            }
            pv.v[0] = dj;
            pv.v[1] = dx;
            pv.v[2] = dtr;
            pv.v[3] = (double)acl;
        } else {
            // FP32: a plain tree over the 32 lane sums (each covers one to a few CRUs; the
            // compensated sums start where most terms meet, across the warp partials of a CTA and
            // the CTA partials of a cell), and one REDUX for the ClCh count.  The per-step tree ran
            // on every lane of every warp: with compensation it was ~150 instructions per CRU-step
            // of a 12,500-CRU cell.
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                jh += __shfl_xor_sync(0xffffffffu, jh, o);
                xh += __shfl_xor_sync(0xffffffffu, xh, o);
                th += __shfl_xor_sync(0xffffffffu, th, o);
            }
            acl = (int)__reduce_add_sync(0xffffffffu, (unsigned)acl);
            float *f = reinterpret_cast<float *>(pv.v);
            f[0] = jh; f[1] = 0.f; f[2] = xh; f[3] = 0.f; f[4] = th; f[5] = 0.f;
            f[6] = (float)acl;
            f[7] = 0.f;
        }
        return pv;
    }
};

// A CTA's view of its work item and of the shared-memory layout, rebuilt from the kernel
// arguments by each of the kernel's parts.
template <bool FP64, bool ODE64>
struct CtaView {
    using R = typename std::conditional<FP64, double, float>::type;
    using T = typename std::conditional<ODE64, double, float>::type;
    CtaWork w;
    int nw, warp, lane, ot, n_ssa;
    bool active, leader, ode_thread;
    SsaConsts<R> *cc;
    R *svbuf;
    OdeShared *os;
    OdeProgram *P;
    T *X;
    math64::Tables *M;
    void *svstage;
    Partial *part;
    float2 *rtab;
    int *fq;        // FP64: queue counters [2] (+2 unused), then the queue
    uint32_t mbar;  // shared address of the partials' mbarrier of parity 0 (parity 1 at +8); the
                    // SSA values' mbarriers of parity 0 and 1 at +16 and +24
    TileRec<R> *tile;
    OdeOffsets off;  // for ode_phase

    __device__ __forceinline__ explicit CtaView(const KernelArgs &a) {
        extern __shared__ __align__(16) unsigned char smem[];
        nw = a.ssa_warps;  // SSA warps of a leader CTA; the other CTAs have nw + kOdeWarps
        warp = (int)(threadIdx.x >> 5);
        lane = (int)(threadIdx.x & 31);
        ot = (int)threadIdx.x - nw * 32;  // ODE thread index 0 .. kOdeLanes-1
        w = a.work[blockIdx.x];
        active = w.cell >= 0;
        leader = active && w.rank_in_cell == 0;
        ode_thread = leader && warp >= nw;
        n_ssa = (leader ? nw : nw + kOdeWarps) * 32;  // SSA threads of this CTA
        const SmemLayout L = smem_layout<R, T>(a.tile_cap, a.max_cta_cell);
        cc = reinterpret_cast<SsaConsts<R> *>(smem + L.cc);
        svbuf = reinterpret_cast<R *>(smem + L.sv);
        os = reinterpret_cast<OdeShared *>(smem + L.ode);
        P = reinterpret_cast<OdeProgram *>(smem + L.prog);
        X = reinterpret_cast<T *>(smem + L.x);
        M = reinterpret_cast<math64::Tables *>(smem + L.math);
        svstage = smem + L.svs;
        part = reinterpret_cast<Partial *>(smem + L.part);
        rtab = reinterpret_cast<float2 *>(smem + L.rtab);
        fq = reinterpret_cast<int *>(smem + L.fq);
        mbar = smem_addr(smem + L.mbar);
        tile = reinterpret_cast<TileRec<R> *>(smem + L.tile);
        off = OdeOffsets{(uint32_t)L.prog, (uint32_t)L.x, (uint32_t)L.ode, (uint32_t)L.math, (uint32_t)L.svs};
    }
};

// The leader CTA's ODE warps over a launch: the transcendental phases of the initial state and
// the push of sv[0], then per global step s the wait for and reduction of the warp partials of
// step s-1, the global step s -> s+1 and the push of sv[(s+1)&1], and the carry back to the cell
// block at the end.  A function of its own (not inlined into the kernel), so that its register allocation and
// schedule do not depend on the SSA code.
template <bool FP64, bool ODE64>
__device__ __noinline__ void ode_warps(const KernelArgs &a, uint64_t step0) {
    using T = typename std::conditional<ODE64, double, float>::type;
    using R = typename std::conditional<FP64, double, float>::type;
    const CtaView<FP64, ODE64> v(a);
    const OdeProgram &P = *v.P;
    OdeShared &os = *v.os;
    T *X = v.X;
    const math64::Tables &M = *v.M;
    const int ot = v.ot, lane = v.lane, cell = v.w.cell;
    const int pslot = a.max_cta_cell * kMaxWarps;  // warp partials per parity slot
    {
        // program, constants and state of the cell
        const int4 *src = reinterpret_cast<const int4 *>(a.prog);
        int4 *dst = reinterpret_cast<int4 *>(v.P);
        for (int i = ot; i < (int)(sizeof(OdeProgram) / 16); i += kOdeLanes) dst[i] = src[i];
    }
    {
        const CellStatic &C = a.cs[cell];
        const CellDyn &d = a.dyn[cell];
        for (int i = ot; i < kOdeMaxSlots; i += kOdeLanes) X[i] = (T)0;
        math64::load_tables(*v.M, ot, kOdeLanes);
        ode_bar();
        if (ot == 0) {
            X[XS_ONE] = (T)1;
            X[XS_MONE] = (T)-1;
            os.t = d.t;
            os.sums[0] = d.sum_jlcc;
            os.sums[1] = d.sum_clch;
            os.sums[2] = d.sum_jtr;
            os.sums[3] = d.sum_jxfer;
            os.status = 0;
            X[XS_DT] = (T)a.dt;
            X[XS_ISTIM] = (T)stimulus(d, d.t, a.run_step0);
            for (int i = 0; i < 4; ++i) X[XS_SUMS + i] = (T)os.sums[i];
        }
        for (int i = ot; i < kNumGlobals; i += kOdeLanes) {
            os.g[i] = d.g[i];
            X[XS_G + i] = X[XS_GN + i] = (T)d.g[i];
        }
        for (int i = ot; i < kOdeConstCap; i += kOdeLanes) X[XS_FIRST_FREE + i] = (T)C.ode_consts[i];
        ode_bar();
        // staging row: the constant SSA values once per launch, Cai and CaNSR of the initial state
        // (the other values are staged by the phases that compute them)
        R *stage = reinterpret_cast<R *>(v.svstage);
        if (ot < kSvCount && ot != SV_CAI && ot != SV_CANSR && ot != SV_CAI_LO && ot != SV_CANSR_LO &&
            P.sv_src[ot] < XS_FIRST_FREE + kOdeMaxConsts)
            stage[ot] = (R)X[P.sv_src[ot]];
        if (ot == 0) stage_pair(stage, SV_CAI, SV_CAI_LO, os.g[3]);
        if (ot == 1) stage_pair(stage, SV_CANSR, SV_CANSR_LO, os.g[4]);
    }
    // The next step's stimulus is formed by lane 0 of a warp without ops in the update phase (its
    // t_{s+1} is os.t + dt, the same addition as the update's), else of one idle in the push
    // phase (os.t is then t_{s+1}), else by thread 0 before the push.
    int stim_q = -1, stim_warp = 0;
    for (int w = kOdeWarps - 1; w >= 0; --w)
        if (stim_q < 0 && P.wkind[P.upd_phase][w] == OK_NOP) stim_q = P.upd_phase, stim_warp = w;
    for (int w = kOdeWarps - 1; w >= 0; --w)
        if (stim_q < 0 && P.push_phase > P.upd_phase && P.wkind[P.push_phase][w] == OK_NOP)
            stim_q = P.push_phase, stim_warp = w;
    // transcendental phases of the initial state, push sv[0]
    {
        const int reg = v_regime(os.g[0]);
        for (int q = P.upd_phase + 1; q <= P.push_phase; ++q) {
            ode_phase<T, R>(v.off, q, reg, ot);
            ode_bar();
        }
        // (the SSA warps wait for these bytes in step 0: the host launches 1..steps_per_launch
        // steps, never 0, so no CTA exits while they may be in flight)
        push_sv<FP64>(v.svbuf, v.svstage, 0, v.mbar + 16u, v.w, ot);
        for (int q = P.push_phase + 1; q < P.n_phases; ++q) {
            ode_phase<T, R>(v.off, q, reg, ot);
            ode_bar();
        }
    }
    // bytes of the cell's warp partials per step (every SSA warp of the cell pushes 32 B)
    const uint32_t part_bytes =
        (uint32_t)sizeof(Partial) * (uint32_t)(v.nw + (v.w.n_cta_cell - 1) * (v.nw + kOdeWarps));
    bool stopped = false;  // a wait ran out (the same on every ODE thread)
    int s_stop = -1;       // the step whose wait (for the partials of step s_stop - 1) ran out
    for (int s = 0; s < a.n_steps; ++s) {
        const int par = s & 1;
        const int64_t ri = a.run_step0 + s;
        const bool rec = a.record_every > 0 && (ri % a.record_every) == 0;
        const int64_t r_idx = rec ? ri / a.record_every - a.rec_base : -1;
        const bool rec_ok = rec && r_idx >= 0 && r_idx < a.rec_cap;
        // After a wait has run out the cell stops for the rest of the launch (no waits, no
        // declarations, no pushes): its CTAs then run out their own waits and stop too, so the
        // launch ends within about a second per CTA and few stray bytes land on any mbarrier.
        if (stopped) continue;
        // the partials of step s will complete the next phase of mbarrier par (the previous one,
        // step s-2's, completed before this thread's wait in step s-1)
        if (ot == 0)
            mbar_arrive_expect_tx(v.mbar + 8u * (uint32_t)par,
                                  part_bytes + (s == a.n_steps - 1 ? (uint32_t)a.test_extra_tx : 0u));
        // fluxes of step s-1 (or the carry), then the global step s -> s+1
        if (ot == 0 && (not_positive(os.g[1]) || not_positive(os.g[2])) && os.status == 0)
            os.status = GW_ERR_NERNST;
        if (s > 0) {
            const bool ok = mbar_wait(v.mbar + 8u * (uint32_t)(par ^ 1), (uint32_t)((s - 1) >> 1) & 1u);
            if (bar_or(1, kOdeLanes, !ok)) {  // the same decision on all ODE threads
                if (ot == 0) atomicCAS(&os.status, 0, (int)GW_ERR_SYNC_TIMEOUT);
                stopped = true;
                s_stop = s;
                continue;
            }
        }
        if (s > 0) reduce_partials<FP64, T>(v.part + (par ^ 1) * pslot, v.w.n_cta_cell * kMaxWarps, ot >> 5, lane, os.sums, X);
        if (s > 0 && ot == 0) X[XS_ISTIM] = (T)os.stim[par];  // formed in step s-1 (below)
        ode_bar();
        const int reg_n = v_regime(os.g[0]);
        for (int q = 0; q <= P.upd_phase; ++q) {
            if (q == stim_q && lane == 0 && (ot >> 5) == stim_warp)
                os.stim[par ^ 1] = stimulus(a.dyn[cell], os.t + a.dt, ri + 1);
            ode_phase<T, R>(v.off, q, reg_n, ot);
            ode_bar();
        }
        if (ot == 0) os.t += a.dt;
        if (rec_ok) {
            double *dst = a.tr_glob + ((int64_t)cell * a.rec_cap + r_idx) * kNumGlobals;
            for (int i = ot; i < kNumGlobals; i += kOdeLanes) dst[i] = os.g[i];
            if (ot == 0 && (cell == 0 || (a.tr_cell >= 0 && cell == a.tr_cell))) a.tr_t[r_idx] = os.t;
        }
        const int reg = v_regime(os.g[0]);
        // Cai and CaNSR of the new state with their FP32 remainders, staged for the push by two
        // lanes of the last ODE warp, whose ops in the next phase finish early
        if (ot == kOdeLanes - 1) stage_pair(reinterpret_cast<R *>(v.svstage), SV_CAI, SV_CAI_LO, os.g[3]);
        if (ot == kOdeLanes - 2) stage_pair(reinterpret_cast<R *>(v.svstage), SV_CANSR, SV_CANSR_LO, os.g[4]);
        for (int q = P.upd_phase + 1; q <= P.push_phase; ++q) {
            if (q == stim_q && lane == 0 && (ot >> 5) == stim_warp)
                os.stim[par ^ 1] = stimulus(a.dyn[cell], os.t, ri + 1);
            ode_phase<T, R>(v.off, q, reg, ot);
            ode_bar();
        }
        // (no warp idle in either phase: the stimulus formed here)
        if (stim_q < 0 && ot == 0) os.stim[par ^ 1] = stimulus(a.dyn[cell], os.t, ri + 1);
        // (no push after the launch's last step: no one would wait for those bytes, and a CTA
        // must not exit while stores into its shared memory may still be in flight)
        if (s + 1 < a.n_steps)
            push_sv<FP64>(v.svbuf, v.svstage, par ^ 1, v.mbar + 16u + 8u * (uint32_t)(par ^ 1), v.w, ot);
        // the new globals become the old ones of the next step's increments (read after the
        // next step's ode_bar; no phase after this point reads XS_G)
        if (ot < kNumGlobals) X[XS_G + ot] = X[XS_GN + ot];
        // off the critical path: the phases the SSA does not need
        for (int q = P.push_phase + 1; q < P.n_phases; ++q) {
            ode_phase<T, R>(v.off, q, reg, ot);
            ode_bar();
        }
    }
    // carry of the last step's fluxes, globals and counters back to the cell block
    if (a.n_steps > 0 && !stopped) {
        const bool ok =
            mbar_wait(v.mbar + 8u * (uint32_t)((a.n_steps - 1) & 1), (uint32_t)((a.n_steps - 1) >> 1) & 1u);
        if (bar_or(1, kOdeLanes, !ok) && ot == 0) atomicCAS(&os.status, 0, (int)GW_ERR_SYNC_TIMEOUT);
    }
    // After a wait ran out in step s_stop, warp partials of steps s_stop - 1 and s_stop may still
    // land here (the cell's CTAs send step s + 1 only after the SSA values of step s + 1, which the
    // leader pushes only after the partials of step s - 1): thread 0 waits, bounded, for both
    // declared phases, so that no store into this CTA is in flight when it exits (an st.async
    // completes only on its mbarrier; the closing cluster barrier does not order it).
    if (stopped && ot == 0 && s_stop >= 1) {
        mbar_wait(v.mbar + 8u * (uint32_t)((s_stop - 1) & 1), (uint32_t)((s_stop - 1) >> 1) & 1u);
        mbar_wait(v.mbar + 8u * (uint32_t)(s_stop & 1), (uint32_t)(s_stop >> 1) & 1u);
    }
    if (a.n_steps > 0)
        reduce_partials<FP64, T>(v.part + ((a.n_steps - 1) & 1) * pslot, v.w.n_cta_cell * kMaxWarps, ot >> 5, lane, os.sums, X);
    ode_bar();
    CellDyn &d = a.dyn[cell];
    for (int i = ot; i < kNumGlobals; i += kOdeLanes) d.g[i] = os.g[i];
    if (ot == 0) {
        d.sum_jlcc = os.sums[0];
        d.sum_clch = os.sums[1];
        d.sum_jtr = os.sums[2];
        d.sum_jxfer = os.sums[3];
        d.t = os.t;
        d.step = step0 + (uint64_t)a.n_steps;
        if (os.status != 0) atomicCAS(&a.status[cell], 0, os.status);
    }
    // the launch's one closing cluster barrier (every thread of every CTA of the cluster)
    cluster_arrive();
    cluster_wait();
}

// The SSA warps over a launch (every warp of a CTA that is not a leader's ODE warp, and every
// warp of an idle CTA, which only keeps the closing cluster barrier): per global step the SSA of
// the warp's CRUs, the record pass and the flux partials, and the tile back to the cell's planes
// at the end.  Inlined into the kernel (out of line it spills).
template <bool FP64, bool ODE64>
__device__ __forceinline__ void ssa_warps(const KernelArgs &a, uint64_t step0) {
    using R = typename std::conditional<FP64, double, float>::type;
    constexpr bool EXACT = FP64;
    const CtaView<FP64, ODE64> v(a);
    const CtaWork &w = v.w;
    const int warp = v.warp, lane = v.lane, cell = w.cell, n_ssa = v.n_ssa;
    const SsaConsts<R> &cc = *v.cc;
    TileRec<R> *tile = v.tile;
    const int pslot = a.max_cta_cell * kMaxWarps;  // warp partials per parity slot
    const R dt = (R)a.dt;
    unsigned long long my_events = 0;
    int my_err = 0;  // bit 0: a CRU hit the event cap; bit 1: a wait for the SSA values ran out
    int s_stop = -1;  // the step whose wait ran out
    for (int s = 0; s < a.n_steps; ++s) {
        const int par = s & 1;
        const int64_t ri = a.run_step0 + s;
        const bool rec = a.record_every > 0 && (ri % a.record_every) == 0;
        const int64_t r_idx = rec ? ri / a.record_every - a.rec_base : -1;
        const bool rec_ok = rec && r_idx >= 0 && r_idx < a.rec_cap;
        if (v.active && !(my_err & 2)) {
            // The SSA values of step s arrive by st.async from the leader's ODE warps and complete
            // this CTA's mbarrier of parity par (thread 0 declares the bytes; that mbarrier's
            // previous phase, step s-2's, completed before this CTA's waits of step s-2).  The
            // CTA's SSA threads then meet at named barrier 2 (bar_or below; the CTAs of a cell are
            // held together only by their data) and take the wait's outcome together: after a
            // wait has run out the CTA stops for the rest of the launch (no more sends), so that
            // its partners stop too.
            const uint32_t svm = v.mbar + 16u + 8u * (uint32_t)par;
            if (threadIdx.x == 0) mbar_arrive_expect_tx(svm, (uint32_t)(kSvCount * sizeof(R)));
            const bool ok = mbar_wait(svm, (uint32_t)(s >> 1) & 1u);
            const R *sv = v.svbuf + par * kSvCount;
            // FP32: the CTA's rate table of this step, entry e by SSA thread e, into the table of
            // this parity, before bar_or(2) of step s, which publishes it.  No reader of that
            // table (step s-2's) can remain: every SSA thread passed bar_or of step s-1 after its
            // last iteration of step s-2.  A warp still in step s-1 reads the other table.
            float2 *rtab = v.rtab + par * kRateTab;
            if (!FP64)
                for (int e = (int)threadIdx.x; e < kRateTab; e += n_ssa) build_rate_entry<R>(rtab, cc, sv, e);
            // FP64: float copies of the step's SSA values for the screen, in the same place and
            // under the same rule (floats 0..kSvCount-1 of this parity's table)
            float *svf = reinterpret_cast<float *>(rtab);
            const float *sk = reinterpret_cast<const float *>(v.rtab) + 64;
            if (FP64)
                for (int e = (int)threadIdx.x; e < kSvCount; e += n_ssa) svf[e] = (float)sv[e];
            if (bar_or(2, n_ssa, !ok)) {
                my_err |= 2;
                s_stop = s;
                continue;
            }
            const int nsw = n_ssa >> 5;
            // This warp's CRUs [cursor, end).  A lane whose CRU has finished its step takes the
            // next one, so lanes with pending SSA events do not hold the others back.
            // (a leader takes CRUs on its first lead_warps SSA warps only, possibly none)
            // FP64: no more working warps than ceil(CRUs / 32).  An FP64 warp instruction takes its
            // sub-partition's FP64 pipe for ~64 cycles whatever its active lanes, so two warps of
            // 16 CRUs cost twice one warp of 32; the first warps of a CTA sit on distinct
            // sub-partitions.
            int nse = v.leader ? w.lead_warps : nsw;
            if (FP64) nse = min(nse, (w.cru_count + 31) >> 5);
            const int beg = warp < nse ? (int)((int64_t)w.cru_count * warp / nse) : w.cru_count;
            const int end = warp < nse ? (int)((int64_t)w.cru_count * (warp + 1) / nse) : w.cru_count;
            int cursor = beg;
            FluxAcc<FP64> acc;
            Cru<R> c;
            SsaLane<R, EXACT> sl;
            Stream rng;
            int m = -1;  // CRU of this lane; -1 none yet, -2 none left
            if constexpr (FP64) {
                // Pass 1: the warp's CRUs, one iteration per lane and pass.  An iteration that the
                // FP32 screen shows to be the step's last runs without the FP64 rates (finish); a
                // CRU whose first iteration it declines (an event in the step) goes, untouched in
                // the tile, to the CTA's queue, and its lane takes the next CRU.
                int *qn = v.fq + par;
                int *q = v.fq + 4;
                if (threadIdx.x == 0) v.fq[par ^ 1] = 0;  // step s-1's count: every reader has passed
                                                          // bar_or(2) of this step
                bool fresh = false;
                for (;;) {
                    const unsigned need = __ballot_sync(0xffffffffu, m == -1);
                    if (need) {
                        const int nm = cursor + __popc(need & ((1u << lane) - 1u));
                        cursor += __popc(need);
                        if (m == -1) {
                            if (nm < end) {
                                m = nm;
                                tile_get(c, tile[m]);
                                rng.open(a.seed, (uint32_t)(a.cell_base + cell), (uint32_t)(w.cru_begin + m),
                                         step0 + s, 0);
                                sl.begin(c, cc);
                                fresh = true;
                            } else {
                                m = -2;
                            }
                        }
                    }
                    if (!__any_sync(0xffffffffu, m >= 0)) break;
                    if (m >= 0) {
                        int err = 0;
                        bool done = false;
                        if (sl.surely_last(c, cc, sk, svf, rng, dt)) {
                            sl.finish(c, cc, sv, rng, dt);
                            done = true;
                        } else {
                            const int qs = fresh ? atomicAdd(qn, 1) : kEngQCap;
                            if (qs < kEngQCap) {
                                q[qs] = m;
                                m = -1;
                            } else {  // the queue is full, or the CRU is past its first iteration
                                done = sl.iterate(c, cc, sv, rtab, rng, dt, a.event_cap, err);
                            }
                        }
                        fresh = false;
                        if (done) {
                            tile_put(tile[m], c);
                            my_events += (unsigned long long)sl.ev;
                            my_err |= err;
                            acc.add(c.jlcc[0] + c.jlcc[1] + c.jlcc[2] + c.jlcc[3], sl.jxfer_sum, sl.jtr,
                                    __popc((c.flags >> 4) & 0xFu));
                            m = -1;
                        }
                    }
                }
                // Pass 2: the queued CRUs on four lanes each (SsaLane::iterate_group: one subunit's
                // rates per lane), eight per warp at a time, over the CTA's SSA warps.
                ssa_bar(n_ssa);
                const int nq = min(*qn, kEngQCap);
                const int jq = lane & 3, base = lane & ~3;
                const int nwu = min(nsw, (nq + 7) >> 3);
                if (warp < nwu) {
                    int qc = (int)((int64_t)nq * warp / nwu);
                    const int qe = (int)((int64_t)nq * (warp + 1) / nwu);
                    m = -1;
                    bool first = false;
                    for (;;) {
                        const unsigned need = __ballot_sync(0xffffffffu, m == -1 && jq == 0);
                        if (need) {
                            const int nm = qc + __popc(need & ((1u << base) - 1u));
                            qc += __popc(need);
                            if (m == -1) {
                                if (nm < qe) {
                                    m = q[nm];
                                    tile_get(c, tile[m]);
                                    rng.open(a.seed, (uint32_t)(a.cell_base + cell), (uint32_t)(w.cru_begin + m),
                                             step0 + s, 0);
                                    sl.begin(c, cc);
                                    first = true;
                                } else {
                                    m = -2;
                                }
                            }
                        }
                        if (!__any_sync(0xffffffffu, m >= 0)) break;
                        if (m >= 0) {
                            int err = 0;
                            bool done;
                            if (!first && sl.surely_last(c, cc, sk, svf, rng, dt)) {
                                sl.finish(c, cc, sv, rng, dt);
                                done = true;
                            } else {
                                done = sl.iterate_group(c, cc, sv, rng, dt, a.event_cap, err);
                            }
                            first = false;
                            if (done) {
                                if (jq == 0) {
                                    tile_put(tile[m], c);
                                    my_events += (unsigned long long)sl.ev;
                                    my_err |= err;
                                    acc.add(c.jlcc[0] + c.jlcc[1] + c.jlcc[2] + c.jlcc[3], sl.jxfer_sum, sl.jtr,
                                            __popc((c.flags >> 4) & 0xFu));
                                }
                                m = -1;
                            }
                        }
                    }
                }
                // the records read the warps' tile ranges, which pass 2 may have written elsewhere
                if (rec_ok && (cell == a.tr_cell || a.tr_sums != nullptr)) ssa_bar(n_ssa);
            } else {
                for (;;) {
                    const unsigned need = __ballot_sync(0xffffffffu, m == -1);
                    if (need) {
                        const int nm = cursor + __popc(need & ((1u << lane) - 1u));
                        cursor += __popc(need);
                        if (m == -1) {
                            if (nm < end) {
                                m = nm;
                                tile_get(c, tile[m]);
                                rng.open(a.seed, (uint32_t)(a.cell_base + cell), (uint32_t)(w.cru_begin + m),
                                         step0 + s, 0);
                                sl.begin(c, cc);
                            } else {
                                m = -2;
                            }
                        }
                    }
                    if (!__any_sync(0xffffffffu, m >= 0)) break;
                    if (m >= 0) {
                        int err = 0;
                        if (sl.iterate(c, cc, sv, rtab, rng, dt, a.event_cap, err)) {
                            tile_put(tile[m], c);
                            my_events += (unsigned long long)sl.ev;
                            my_err |= err;
                            acc.add(c.jlcc[0] + c.jlcc[1] + c.jlcc[2] + c.jlcc[3], sl.jxfer_sum, sl.jtr,
                                    __popc((c.flags >> 4) & 0xFu));
                            m = -1;
                        }
                    }
                }
            }
            // Records of this step, from the warp's part of the tile (now at the end of the step)
            if (rec_ok && (cell == a.tr_cell || a.tr_sums != nullptr))
                record_pass<R>(a, w, cell, r_idx, beg, end, lane, tile);
            // The warp partial, pushed straight into the leader's slot (rank, warp): the leader
            // sums the cell's warp partials in slot order (no reduction on this side).
            const Partial pv = acc.warp_total();
            if (lane == 0) {
                // two 16-byte asynchronous stores that count themselves off the leader's mbarrier
                // of this parity (the warp goes on without waiting for them to land)
                Partial *dst = v.part + par * pslot + w.rank_in_cell * kMaxWarps + warp;
                const uint32_t rd = map_rank(dst, (uint32_t)w.first);
                const uint32_t rm = map_rank_addr(v.mbar + 8u * (uint32_t)par, (uint32_t)w.first);
                st_async(rd, make_uint4(lo_of(pv.v[0]), hi_of(pv.v[0]), lo_of(pv.v[1]), hi_of(pv.v[1])), rm);
                st_async(rd + 16u, make_uint4(lo_of(pv.v[2]), hi_of(pv.v[2]), lo_of(pv.v[3]), hi_of(pv.v[3])), rm);
            }
        }
    }
    // A CTA that stopped at step s_stop may still receive the SSA values of steps s_stop and
    // s_stop + 1, stores the leader issued before it stopped in turn (it pushes step s + 2 only
    // after this CTA's partials of step s, which a stopped CTA does not send).  Nothing orders the
    // landing of an st.async with the closing cluster barrier; its completion shows only on the
    // receiving mbarrier.  So thread 0 waits, bounded, for those two phases before the barrier
    // (declaring the bytes of step s_stop + 1, whose phase was not declared yet): no store into
    // this CTA's shared memory is in flight when it exits.
    if ((my_err & 2) && threadIdx.x == 0 && s_stop >= 0) {
        const uint32_t m0 = v.mbar + 16u + 8u * (uint32_t)(s_stop & 1);
        mbar_wait(m0, (uint32_t)(s_stop >> 1) & 1u);
        if (s_stop + 1 < a.n_steps) {
            const uint32_t m1 = v.mbar + 16u + 8u * (uint32_t)((s_stop + 1) & 1);
            mbar_arrive_expect_tx(m1, (uint32_t)(kSvCount * sizeof(R)));
            mbar_wait(m1, (uint32_t)((s_stop + 1) >> 1) & 1u);
        }
    }
    // the launch's one closing cluster barrier (every thread of every CTA of the cluster)
    cluster_arrive();
    cluster_wait();
    if (!v.active) return;
    // the tile back to the cell's planes
    R *g_cass = reinterpret_cast<R *>(a.cass);
    R *g_jlcc = reinterpret_cast<R *>(a.jlcc);
    R *g_cajsr = reinterpret_cast<R *>(a.cajsr);
    const int64_t base = a.slot0[cell] + w.cru_begin;
    for (int m = (int)threadIdx.x; m < w.cru_count; m += n_ssa) {
        const int64_t gs = base + m;
        Cru<R> c;
        tile_get(c, tile[m]);
        a.lcc[gs] = c.lcc;
        a.flags[gs] = c.flags;
#pragma unroll
        for (int k = 0; k < 6; ++k) a.ryr[k * a.n_slots + gs] = c.ryr[k];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            g_cass[j * a.n_slots + gs] = c.cass[j];
            g_jlcc[j * a.n_slots + gs] = c.jlcc[j];
        }
        g_cajsr[gs] = c.cajsr;
        if (!FP64) a.cajsr_lo[gs] = c.cajsr_lo;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        my_events += __shfl_xor_sync(0xffffffffu, my_events, o);
        my_err |= __shfl_xor_sync(0xffffffffu, my_err, o);
    }
    if (lane == 0) {
        if (my_events) atomicAdd(a.events, my_events);
        if (my_err) atomicCAS(&a.status[cell], 0, (my_err & 2) ? (int)GW_ERR_SYNC_TIMEOUT : (int)GW_ERR_EVENT_CAP);
    }
}

// The engine kernel: every CTA of a cluster initialises its mbarriers and waits for the whole
// cluster to be resident (it writes into the other CTAs' shared memory from its first global step
// on), loads its CRU tile and the cell's SSA constants, then splits into the ODE warps of a leader
// CTA and the SSA warps.  Both parts end with one more cluster barrier, so that no CTA exits
// while another may still write into its shared memory.
template <bool FP64, bool ODE64>
__global__ void __launch_bounds__(FP64 ? kMaxThreadsFp64 : kMaxThreads, 1) engine_kernel(const __grid_constant__ KernelArgs a) {
    using R = typename std::conditional<FP64, double, float>::type;
    const CtaView<FP64, ODE64> v(a);
    // The partials' mbarriers (one arrival per phase: the ODE thread's expect_tx) are initialised
    // before the cluster barrier that every CTA passes before its first remote write.
    if (threadIdx.x == 0) {
        for (uint32_t i = 0; i < 4; ++i) mbar_init(v.mbar + 8u * i, 1);
        mbar_fence_init();
    }
    cluster_arrive();
    cluster_wait();
    uint64_t step0 = 0;
    if (v.active) {
        const int cell = v.w.cell;
        if (threadIdx.x == 0) {
            load_ssa_consts<R>(*v.cc, a.cs[cell]);
            // FP64: the screen's constants (SsaLane::surely_last) in the rate-table area, which the
            // FP64 lane does not otherwise use: floats 64.. of parity 0's table
            if (FP64) {
                load_screen_consts(reinterpret_cast<float *>(v.rtab) + 64, a.cs[cell]);
                v.fq[0] = 0;
                v.fq[1] = 0;
            }
        }
        // The leader's warp-partial slots start at zero (slots of warps a CTA does not have stay
        // so); the cell's CTAs write them only after the first cluster barrier of the steps.
        if (v.leader) {
            double *pz = &v.part[0].v[0];
            const int nz = 2 * a.max_cta_cell * kMaxWarps * 4;
            for (int i = (int)threadIdx.x; i < nz; i += (int)blockDim.x) pz[i] = 0.0;
        }
        step0 = a.dyn[cell].step;
        if (!v.ode_thread) {
            R *g_cass = reinterpret_cast<R *>(a.cass);
            R *g_jlcc = reinterpret_cast<R *>(a.jlcc);
            R *g_cajsr = reinterpret_cast<R *>(a.cajsr);
            const int64_t base = a.slot0[cell] + v.w.cru_begin;
            for (int m = (int)threadIdx.x; m < v.w.cru_count; m += v.n_ssa) {
                const int64_t gs = base + m;
                Cru<R> c;
                c.lcc = a.lcc[gs];
                c.flags = a.flags[gs];
#pragma unroll
                for (int k = 0; k < 6; ++k) c.ryr[k] = a.ryr[k * a.n_slots + gs];
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    c.cass[j] = g_cass[j * a.n_slots + gs];
                    c.jlcc[j] = g_jlcc[j * a.n_slots + gs];
                }
                c.cajsr = g_cajsr[gs];
                c.cajsr_lo = FP64 ? 0.f : a.cajsr_lo[gs];
                tile_put(v.tile[m], c);
            }
        }
    }
    __syncthreads();
    if (v.ode_thread)
        ode_warps<FP64, ODE64>(a, step0);
    else
        ssa_warps<FP64, ODE64>(a, step0);
}

// Random initial CRU state (GW_utils.tpp:5-64) from stream 1, one thread per CRU, in the same
// draw order as the oracle's orc_sample_initial_crus.
template <bool FP64>
__global__ void init_crus_kernel(const KernelArgs a, int cell, int ncru) {
    using R = typename std::conditional<FP64, double, float>::type;
    const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (i >= ncru) return;
    Stream s;
    s.open(a.seed, (uint32_t)(a.cell_base + cell), (uint32_t)i, 0, 1);
    uint32_t k = 0;
    auto pick = [&](const double *w, int n) {
        const double u = FP64 ? s.u53(k) : (double)s.u24(k);
        ++k;
        double cum = w[0];
        int idx = 0;
        while (cum < u && idx < n - 1) {
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

template <bool FP64, bool ODE64>
inline cudaError_t set_attrs(size_t smem) {
    auto k = engine_kernel<FP64, ODE64>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    return e;
}

inline cudaLaunchConfig_t launch_cfg(const LaunchShape &s, void *stream, cudaLaunchAttribute *attr) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)s.ctas, 1, 1);
    cfg.blockDim = dim3((unsigned)s.threads, 1, 1);
    cfg.dynamicSmemBytes = s.smem;
    cfg.stream = (cudaStream_t)stream;
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)s.cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cfg;
}

template <bool FP64>
inline int launch_engine(const KernelArgs &a, const LaunchShape &s, void *stream, bool ode64) {
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t cfg = launch_cfg(s, stream, attr);
    cudaError_t e;
    if constexpr (FP64) {
        (void)ode64;
        e = set_attrs<true, true>(s.smem);
        if (e == cudaSuccess) e = cudaLaunchKernelEx(&cfg, engine_kernel<true, true>, a);
    } else if (ode64) {
        e = set_attrs<false, true>(s.smem);
        if (e == cudaSuccess) e = cudaLaunchKernelEx(&cfg, engine_kernel<false, true>, a);
    } else {
        e = set_attrs<false, false>(s.smem);
        if (e == cudaSuccess) e = cudaLaunchKernelEx(&cfg, engine_kernel<false, false>, a);
    }
    return (int)e;
}

template <bool FP64>
inline int max_active_clusters(const LaunchShape &s, bool ode64, int *out) {
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t cfg = launch_cfg(s, nullptr, attr);
    cudaError_t e;
    if constexpr (FP64) {
        (void)ode64;
        e = set_attrs<true, true>(s.smem);
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveClusters(out, engine_kernel<true, true>, &cfg);
    } else if (ode64) {
        e = set_attrs<false, true>(s.smem);
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveClusters(out, engine_kernel<false, true>, &cfg);
    } else {
        e = set_attrs<false, false>(s.smem);
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveClusters(out, engine_kernel<false, false>, &cfg);
    }
    return (int)e;
}

}  // namespace dev
}  // namespace gw
