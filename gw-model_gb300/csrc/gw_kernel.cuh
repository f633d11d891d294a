// gw_kernel.cuh -- the per-CRU hybrid SSA of the GB300 engine (device functions; the engine
// kernel that runs them is in gw_engine.cuh).
//
// One launch advances every cell of an ensemble by n_steps global steps.  A cell's CRUs are
// spread over the CTAs of one thread-block cluster; each CTA keeps its CRU tile in shared memory
// for the whole launch (no HBM traffic per step).  Per global step n:
//
//   SSA warps   : per-CRU hybrid SSA of step n (SSA.tpp:286-310) with V, Cai, CaNSR of step n,
//                 then per-warp flux partials pushed into the leader CTA's shared memory (DSMEM).
//   ODE warps   : (the four last warps of each cell's leader CTA, concurrently with the SSA warps)
//                 reduce the partials of step n-1 and take the FP64 global step n -> n+1
//                 (GW.tpp:237-272), then push the per-step SSA values of step n+1 to every CTA
//                 of the cell.
//   No cluster barrier inside a launch: the step's data travel by st.async into double-buffered
//   slots and complete the receiver's mbarrier of that slot (bounded waits).
//
// The reference's ordering is preserved: the global derivatives of step n use the fluxes left by
// the SSA of step n-1 (GW.tpp:188-198) and the SSA of step n uses the globals of step n.
//
// Precision.  FP64 (EXACT): reference expression order, FP64 everywhere, 53-bit uniforms; with
// -fmad=false it reproduces the oracle to rounding of the transcendental functions.  FP32: CRU
// state and propensities in FP32 with 24-bit uniforms, compensated Cai/CaNSR/CaJSR differences,
// direct RyR totals and zero-weight guards in the transition scans (see ssa_cru).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "gw_internal.h"

namespace gw {
namespace dev {

constexpr double kFaraday = 96.5;  // common.hpp:9

// ------------------------------------------------------------------------------------------
// Counter-based uniforms: Philox4x32-10 (Salmon et al., SC'11), key {seed_lo, seed_hi},
// counter {draw >> 1, cru, step, (stream << 28) | cell}; draw k uses 64-bit lane pair k & 1.
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ void philox10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                         uint32_t k0, uint32_t k1, uint32_t out[4]) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
        const uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
        const uint32_t n0 = hi1 ^ c1 ^ k0;
        const uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

struct Stream {
    uint32_t k0, k1, cru, step, cellw;
    uint32_t blk;
    uint32_t b[4];
    __device__ __forceinline__ void open(uint64_t seed, uint32_t cell, uint32_t cru_, uint64_t step_,
                                         uint32_t stream) {
        k0 = (uint32_t)seed;
        k1 = (uint32_t)(seed >> 32);
        cru = cru_;
        step = (uint32_t)step_;
        cellw = (stream << 28) | (cell & 0x0FFFFFFFu);
        blk = 0xFFFFFFFFu;
    }
    __device__ __forceinline__ void words(uint32_t k, uint32_t &hi, uint32_t &lo) {
        const uint32_t want = k >> 1;
        if (want != blk) {
            philox10(want, cru, step, cellw, k0, k1, b);
            blk = want;
        }
        const bool h = (k & 1u) != 0;
        hi = h ? b[3] : b[1];
        lo = h ? b[2] : b[0];
    }
    // U53: max(w >> 11, 1) * 2^-53
    __device__ __forceinline__ double u53(uint32_t k) {
        uint32_t hi, lo;
        words(k, hi, lo);
        unsigned long long m = ((((unsigned long long)hi) << 32) | lo) >> 11;
        if (m == 0ull) m = 1ull;
        return (double)m * 0x1p-53;
    }
    // U24: max(w >> 40, 1) * 2^-24  (exact in float)
    __device__ __forceinline__ float u24(uint32_t k) {
        uint32_t hi, lo;
        words(k, hi, lo);
        uint32_t m = hi >> 8;
        if (m == 0u) m = 1u;
        return (float)m * 0x1p-24f;
    }
    template <typename R>
    __device__ __forceinline__ R uniform(uint32_t k);
    // U24 draws k, k+1, k+2 (an event selection's draws).  They lie in blocks k >> 1 and
    // (k >> 1) + 1; both are computed without a branch, so that their rounds interleave (the first
    // is often the block already held: recomputing it costs instructions but no latency), and the
    // second is kept for the next draws.
    __device__ __forceinline__ void u24x3(uint32_t k, float &a, float &b2, float &c) {
        const uint32_t B = k >> 1;
        uint32_t o1[4], o2[4];
        philox10(B, cru, step, cellw, k0, k1, o1);
        philox10(B + 1u, cru, step, cellw, k0, k1, o2);
        const bool odd = (k & 1u) != 0u;
        a = u24_of(odd ? o1[3] : o1[1]);
        b2 = u24_of(odd ? o2[1] : o1[3]);
        c = u24_of(odd ? o2[3] : o2[1]);
        blk = B + 1u;
        b[0] = o2[0];
        b[1] = o2[1];
        b[2] = o2[2];
        b[3] = o2[3];
    }
    __device__ __forceinline__ static float u24_of(uint32_t hi) {
        uint32_t m = hi >> 8;
        if (m == 0u) m = 1u;
        return (float)m * 0x1p-24f;
    }
};
template <>
__device__ __forceinline__ double Stream::uniform<double>(uint32_t k) {
    return u53(k);
}
template <>
__device__ __forceinline__ float Stream::uniform<float>(uint32_t k) {
    return u24(k);
}

// ------------------------------------------------------------------------------------------
// Cluster helpers (inline PTX).
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t cluster_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ void cluster_sync() {
    asm volatile("barrier.cluster.arrive.release;\n\tbarrier.cluster.wait.acquire;" ::: "memory");
}
__device__ __forceinline__ uint32_t map_rank(const void *p, uint32_t rank) {
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
    return r;
}
// shared::cluster address of a local shared address (a 32-bit shared-window address) in CTA rank
__device__ __forceinline__ uint32_t map_rank_addr(uint32_t a, uint32_t rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
    return r;
}
__device__ __forceinline__ void st_remote(uint32_t addr, double v) {
    asm volatile("st.shared::cluster.f64 [%0], %1;" ::"r"(addr), "d"(v) : "memory");
}
__device__ __forceinline__ void st_remote(uint32_t addr, float v) {
    asm volatile("st.shared::cluster.f32 [%0], %1;" ::"r"(addr), "f"(v) : "memory");
}
__device__ __forceinline__ void st_remote(uint32_t addr, uint4 v) {  // addr 16-byte aligned
    asm volatile("st.shared::cluster.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(v.x), "r"(v.y), "r"(v.z),
                 "r"(v.w)
                 : "memory");
}

// mbarriers (shared-memory arrival/transaction barriers) and asynchronous remote stores.  An
// st.async writes 16 bytes into a CTA of the cluster and, once the bytes are there, counts them off
// that CTA's mbarrier (complete_tx); the issuing thread does not wait for it, and a later fence
// or release arrive of that thread does not either.  addr and mbar are shared::cluster addresses
// (map_rank), addr 16-byte aligned.
__device__ __forceinline__ void st_async(uint32_t addr, uint4 v, uint32_t mbar) {
    asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v4.b32 [%0], {%1, %2, %3, %4}, [%5];" ::"r"(addr),
                 "r"(v.x), "r"(v.y), "r"(v.z), "r"(v.w), "r"(mbar)
                 : "memory");
}
__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count) : "memory");
}
// makes the initialisations visible to the cluster (before the cluster barrier that precedes
// their first remote use)
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
// one arrival on the local mbarrier, declaring tx more bytes to come in its current phase
__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t mbar, uint32_t tx) {
    uint64_t state;
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 %0, [%1], %2;" : "=l"(state) : "r"(mbar), "r"(tx) : "memory");
    (void)state;
}
// true once the phase of the given parity has completed; acquire at cluster scope, so the bytes
// that completed it (written by other CTAs) are visible.  May suspend the thread for a while.
__device__ __forceinline__ bool mbar_try_wait(uint32_t mbar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(mbar), "r"(parity)
        : "memory");
    return ok != 0u;
}
// Bounded wait: false if the phase did not complete within 2^31 cycles (about a second).
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
    if (mbar_try_wait(mbar, parity)) return true;
    const long long t0 = clock64();
    while (!mbar_try_wait(mbar, parity))
        if (clock64() - t0 > (1ll << 31)) return false;
    return true;
}

// ------------------------------------------------------------------------------------------
// Per-cell SSA constants (shared memory, in the CRU arithmetic type).
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t lcc_table(int s);
__device__ __forceinline__ int lcc_next(int s, int tr);

// Constants of the FP32 lane's packed arithmetic (SsaConsts::pk).
enum PackedConst {
    PK_RISS, PK_M2, PK_RXFER, PK_RRYR, PK_BIAS, PK_K12, PK_K2325, PK_K21, PK_K34, PK_K4543, PK_K32, PK_K45K34,
    PK_K32K43, PK_K43, PK_K5654, PK_K52, PK_K65, PK_K54, PK_K56, PK_KBSR, PK_KBSL, PK_BSR, PK_BSL, PK_COUNT
};

template <typename R>
struct SsaConsts {
    R k12, k21, k23, k32, k34, k43, k45, k54, k56, k65, k25, k52;
    R rRyR, rxfer, rtr, riss, KBSR, KBSL, KCSQN, kfClCh, kbClCh;
    R BSR_const, BSL_const, VSS_VJSR, CSQN_const, Cao_scaled;
    R gam[5];  // gamma0 * a^k, k = 0..4 (Constants gamma0 .. gamma0a4)
    R k2325, k45k34, k32k43, k4543, k5654;  // combined rate constants (FP32 subunit total)
    uint32_t lcct[16];  // LCC rate table by state (lcc_word), in shared memory: no divergent branch
    uint32_t lccn[16];  // next LCC state by state: transition t in bits 4t..4t+3
    float2 pk[PK_COUNT];  // FP32 lane: constants duplicated into (value, value) pairs
};

template <typename R>
__device__ void load_ssa_consts(SsaConsts<R> &c, const CellStatic &s) {
    const gw_params &p = s.p;
    c.k12 = (R)p.k12; c.k21 = (R)p.k21; c.k23 = (R)p.k23; c.k32 = (R)p.k32;
    c.k34 = (R)p.k34; c.k43 = (R)p.k43; c.k45 = (R)p.k45; c.k54 = (R)p.k54;
    c.k56 = (R)p.k56; c.k65 = (R)p.k65; c.k25 = (R)p.k25; c.k52 = (R)p.k52;
    c.rRyR = (R)p.rRyR; c.rxfer = (R)p.rxfer; c.rtr = (R)p.rtr; c.riss = (R)p.riss;
    c.KBSR = (R)p.KBSR; c.KBSL = (R)p.KBSL; c.KCSQN = (R)p.KCSQN;
    c.kfClCh = (R)p.kfClCh; c.kbClCh = (R)p.kbClCh;
    c.BSR_const = (R)s.BSR_const; c.BSL_const = (R)s.BSL_const; c.VSS_VJSR = (R)s.VSS_VJSR;
    c.CSQN_const = (R)s.CSQN_const; c.Cao_scaled = (R)s.Cao_scaled;
    c.gam[0] = (R)s.gamma0; c.gam[1] = (R)s.gamma0a; c.gam[2] = (R)s.gamma0a2;
    c.gam[3] = (R)s.gamma0a3; c.gam[4] = (R)s.gamma0a4;
    c.k2325 = (R)(p.k23 + p.k25);
    c.k45k34 = (R)(p.k45 * p.k34);
    c.k32k43 = (R)(p.k32 * p.k43);
    c.k4543 = (R)(p.k45 + p.k43);
    c.k5654 = (R)(p.k56 + p.k54);
    const float pv[PK_COUNT] = {(float)p.riss, -2.f, (float)p.rxfer, (float)p.rRyR, -8388736.f, (float)p.k12,
                                (float)(p.k23 + p.k25), (float)p.k21, (float)p.k34, (float)(p.k45 + p.k43),
                                (float)p.k32, (float)(p.k45 * p.k34), (float)(p.k32 * p.k43), (float)p.k43,
                                (float)(p.k56 + p.k54), (float)p.k52, (float)p.k65, (float)p.k54, (float)p.k56,
                                (float)p.KBSR, (float)p.KBSL, (float)s.BSR_const, (float)s.BSL_const};
    for (int i = 0; i < PK_COUNT; ++i) c.pk[i] = make_float2(pv[i], pv[i]);
    for (int st = 0; st < 16; ++st) {
        c.lcct[st] = lcc_table(st);
        c.lccn[st] = (uint32_t)lcc_next(st, 0) | ((uint32_t)lcc_next(st, 1) << 4) | ((uint32_t)lcc_next(st, 2) << 8);
    }
}

// LCC transition table: for state s (1..12) the sv[] index of each of its 3 outgoing rates
// (update_LCC_rates, GW_utils.tpp:118-186) in bytes 0..2, and in byte 3 the rate slot that is
// gamma*CaSS (Ca-dependent inactivation, states 1..5) or 3 if none.
__host__ __device__ constexpr uint32_t lcc_word(int i0, int i1, int i2, int kin) {
    return (uint32_t)i0 | ((uint32_t)i1 << 8) | ((uint32_t)i2 << 16) | ((uint32_t)kin << 24);
}
__device__ __forceinline__ uint32_t lcc_table(int s) {
    switch (s) {
    case 1: return lcc_word(SV_A4, SV_ZERO, SV_ZERO, 1);
    case 2: return lcc_word(SV_B1, SV_A3, SV_ZERO, 2);
    case 3: return lcc_word(SV_B2, SV_A2, SV_ZERO, 2);
    case 4: return lcc_word(SV_B3, SV_A1, SV_ZERO, 2);
    case 5: return lcc_word(SV_B4, SV_F, SV_ZERO, 2);
    case 6: return lcc_word(SV_G, SV_ZERO, SV_ZERO, 3);
    case 7: return lcc_word(SV_OM, SV_A4a, SV_ZERO, 3);
    case 8: return lcc_word(SV_OMB1, SV_B1bi, SV_A3a, 3);
    case 9: return lcc_word(SV_OMB2, SV_B2bi, SV_A2a, 3);
    case 10: return lcc_word(SV_OMB3, SV_B3bi, SV_A1a, 3);
    case 11: return lcc_word(SV_OMB4, SV_B4bi, SV_F1, 3);
    case 12: return lcc_word(SV_G1, SV_ZERO, SV_ZERO, 3);
    default: return lcc_word(SV_ZERO, SV_ZERO, SV_ZERO, 3);
    }
}
// Next state of sample_LCC (SSA.tpp:103-197) for transition index tr from state s.
__device__ __forceinline__ int lcc_next(int s, int tr) {
    switch (s) {
    case 1: return tr == 0 ? 2 : 7;
    case 2: return tr == 0 ? 1 : (tr == 1 ? 3 : 8);
    case 3: return tr == 0 ? 2 : (tr == 1 ? 4 : 9);
    case 4: return tr == 0 ? 3 : (tr == 1 ? 5 : 10);
    case 5: return tr == 0 ? 4 : (tr == 1 ? 6 : 11);
    case 6: return 5;
    case 7: return tr == 0 ? 1 : 8;
    case 8: return tr == 0 ? 2 : (tr == 1 ? 7 : 9);
    case 9: return tr == 0 ? 3 : (tr == 1 ? 8 : 10);
    case 10: return tr == 0 ? 4 : (tr == 1 ? 9 : 11);
    case 11: return tr == 0 ? 5 : (tr == 1 ? 10 : 12);
    case 12: return 11;
    default: return s;
    }
}

// ------------------------------------------------------------------------------------------
// CRU state in registers.
// ------------------------------------------------------------------------------------------
template <typename R>
struct Cru {
    uint32_t lcc;     // byte j: LCC state of subunit j
    uint32_t flags;   // bit j: LCC_inactivation, bit 4+j: ClCh
    uint32_t ryr[6];  // plane k byte j: count in state k+1
    R cass[4];
    R jlcc[4];
    R cajsr;
    float cajsr_lo;   // FP32: compensation term of CaJSR
};

// Shared-memory tile record of one CRU: the Cru fields in 16-byte words, so that a lane moves its
// CRU with 5 (FP32) or 7 (FP64) 16-byte accesses instead of 18 scalar ones (the SSA warps' share
// of the shared-memory pipe, which the global step's shuffles and loads also queue on).
//   words 0-1: lcc, flags, ryr[0..5]
//   FP32: 2 cass[0..3], 3 jlcc[0..3], 4 {cajsr, cajsr_lo, 0, 0}
//   FP64: 2-3 cass (lo, hi word pairs), 4-5 jlcc, 6 {cajsr lo, hi, cajsr_lo, 0}
template <typename R>
struct alignas(16) TileRec {
    uint4 w[sizeof(R) == 8 ? 7 : 5];
};

__device__ __forceinline__ void tile_get(Cru<float> &c, const TileRec<float> &t) {
    const uint4 a = t.w[0], b = t.w[1], d = t.w[2], e = t.w[3], f = t.w[4];
    c.lcc = a.x; c.flags = a.y; c.ryr[0] = a.z; c.ryr[1] = a.w;
    c.ryr[2] = b.x; c.ryr[3] = b.y; c.ryr[4] = b.z; c.ryr[5] = b.w;
    c.cass[0] = __uint_as_float(d.x); c.cass[1] = __uint_as_float(d.y);
    c.cass[2] = __uint_as_float(d.z); c.cass[3] = __uint_as_float(d.w);
    c.jlcc[0] = __uint_as_float(e.x); c.jlcc[1] = __uint_as_float(e.y);
    c.jlcc[2] = __uint_as_float(e.z); c.jlcc[3] = __uint_as_float(e.w);
    c.cajsr = __uint_as_float(f.x); c.cajsr_lo = __uint_as_float(f.y);
}
__device__ __forceinline__ void tile_put(TileRec<float> &t, const Cru<float> &c) {
    t.w[0] = make_uint4(c.lcc, c.flags, c.ryr[0], c.ryr[1]);
    t.w[1] = make_uint4(c.ryr[2], c.ryr[3], c.ryr[4], c.ryr[5]);
    t.w[2] = make_uint4(__float_as_uint(c.cass[0]), __float_as_uint(c.cass[1]), __float_as_uint(c.cass[2]),
                        __float_as_uint(c.cass[3]));
    t.w[3] = make_uint4(__float_as_uint(c.jlcc[0]), __float_as_uint(c.jlcc[1]), __float_as_uint(c.jlcc[2]),
                        __float_as_uint(c.jlcc[3]));
    t.w[4] = make_uint4(__float_as_uint(c.cajsr), __float_as_uint(c.cajsr_lo), 0u, 0u);
}
__device__ __forceinline__ double dbl_of(uint32_t lo, uint32_t hi) { return __hiloint2double((int)hi, (int)lo); }
__device__ __forceinline__ uint32_t lo_of(double x) { return (uint32_t)__double2loint(x); }
__device__ __forceinline__ uint32_t hi_of(double x) { return (uint32_t)__double2hiint(x); }
__device__ __forceinline__ void tile_get(Cru<double> &c, const TileRec<double> &t) {
    const uint4 a = t.w[0], b = t.w[1], d0 = t.w[2], d1 = t.w[3], e0 = t.w[4], e1 = t.w[5], f = t.w[6];
    c.lcc = a.x; c.flags = a.y; c.ryr[0] = a.z; c.ryr[1] = a.w;
    c.ryr[2] = b.x; c.ryr[3] = b.y; c.ryr[4] = b.z; c.ryr[5] = b.w;
    c.cass[0] = dbl_of(d0.x, d0.y); c.cass[1] = dbl_of(d0.z, d0.w);
    c.cass[2] = dbl_of(d1.x, d1.y); c.cass[3] = dbl_of(d1.z, d1.w);
    c.jlcc[0] = dbl_of(e0.x, e0.y); c.jlcc[1] = dbl_of(e0.z, e0.w);
    c.jlcc[2] = dbl_of(e1.x, e1.y); c.jlcc[3] = dbl_of(e1.z, e1.w);
    c.cajsr = dbl_of(f.x, f.y); c.cajsr_lo = __uint_as_float(f.z);
}
__device__ __forceinline__ void tile_put(TileRec<double> &t, const Cru<double> &c) {
    t.w[0] = make_uint4(c.lcc, c.flags, c.ryr[0], c.ryr[1]);
    t.w[1] = make_uint4(c.ryr[2], c.ryr[3], c.ryr[4], c.ryr[5]);
    t.w[2] = make_uint4(lo_of(c.cass[0]), hi_of(c.cass[0]), lo_of(c.cass[1]), hi_of(c.cass[1]));
    t.w[3] = make_uint4(lo_of(c.cass[2]), hi_of(c.cass[2]), lo_of(c.cass[3]), hi_of(c.cass[3]));
    t.w[4] = make_uint4(lo_of(c.jlcc[0]), hi_of(c.jlcc[0]), lo_of(c.jlcc[1]), hi_of(c.jlcc[1]));
    t.w[5] = make_uint4(lo_of(c.jlcc[2]), hi_of(c.jlcc[2]), lo_of(c.jlcc[3]), hi_of(c.jlcc[3]));
    t.w[6] = make_uint4(lo_of(c.cajsr), hi_of(c.cajsr), __float_as_uint(c.cajsr_lo), 0u);
}

__device__ __forceinline__ int byte_s(uint32_t w, int j) { return (int)(int8_t)(w >> (8 * j)); }
__device__ __forceinline__ int byte_u(uint32_t w, int j) { return (int)((w >> (8 * j)) & 0xFFu); }
__device__ __forceinline__ uint32_t byte_set(uint32_t w, int j, int v) {
    const uint32_t sh = 8u * (uint32_t)j;
    return (w & ~(0xFFu << sh)) | (((uint32_t)v & 0xFFu) << sh);
}
// per-byte add of d to byte j (no carry across bytes)
__device__ __forceinline__ uint32_t byte_add(uint32_t w, int j, int d) {
    return byte_set(w, j, byte_s(w, j) + d);
}

template <typename R>
struct Rates {      // the outgoing rates of one subunit
    R lcc[3];
    R inact;
    R ryr[12];
    R clch;
};

// update_LCC_rates + update_LCC_inactivation_rates + update_RyR_rates + update_ClCh_rates for
// subunit j (GW_utils.tpp:118-186, 222-255; GW_utils.hpp:378-391); returns the subunit total
// accumulated in the reference's order (update_rates, SSA.tpp:48-56).
template <typename T>
__device__ __forceinline__ T pick4(const T (&a)[4], int i) {
    return i == 0 ? a[0] : (i == 1 ? a[1] : (i == 2 ? a[2] : a[3]));
}

template <typename R>
__device__ __forceinline__ R subunit_rates(const Cru<R> &s, int j, R x, const SsaConsts<R> &c,
                                           const R *sv, Rates<R> &r) {
    const int st = byte_u(s.lcc, j);
    const uint32_t w = c.lcct[st & 15];
    r.lcc[0] = sv[w & 0xFFu];
    r.lcc[1] = sv[(w >> 8) & 0xFFu];
    r.lcc[2] = sv[(w >> 16) & 0xFFu];
    const int kin = (int)(w >> 24);
    if (kin < 3) {
        const R gx = c.gam[st - 1] * x;
        if (kin == 1) r.lcc[1] = gx; else r.lcc[2] = gx;
    }
    r.inact = ((s.flags >> j) & 1u) == 0u ? sv[SV_INACT0] : sv[SV_INACT1];
    const R R0 = (R)byte_s(s.ryr[0], j), R1 = (R)byte_s(s.ryr[1], j), R2 = (R)byte_s(s.ryr[2], j);
    const R R3 = (R)byte_s(s.ryr[3], j), R4 = (R)byte_s(s.ryr[4], j), R5 = (R)byte_s(s.ryr[5], j);
    const R R23 = (R)(byte_s(s.ryr[2], j) + byte_s(s.ryr[3], j));
    const R R45 = (R)(byte_s(s.ryr[4], j) + byte_s(s.ryr[5], j));
    const R x2 = x * x;
    const bool hi34 = x > (R)3.685e-2;
    const bool hi56 = x > (R)1.15e-4;
    r.ryr[0] = R0 * c.k12 * x2;
    r.ryr[1] = R1 * c.k23 * x2;
    r.ryr[2] = R1 * c.k25 * x2;
    r.ryr[6] = R1 * c.k21;
    if (hi34) {
        const R tau34 = (R)1.0 / (c.k34 * x2 + c.k43);
        r.ryr[3] = (R)0;
        r.ryr[4] = R23 * c.k45 * c.k34 * x2 * tau34;
        r.ryr[7] = R23 * c.k32 * c.k43 * tau34;
        r.ryr[8] = (R)0;
    } else {
        r.ryr[3] = R2 * c.k34 * x2;
        r.ryr[4] = R3 * c.k45;
        r.ryr[7] = R2 * c.k32;
        r.ryr[8] = R3 * c.k43;
    }
    if (hi56) {
        const R eq56 = c.k65 / (c.k56 * x2 + c.k65);
        r.ryr[5] = (R)0;
        r.ryr[9] = R45 * c.k52 * eq56;
        r.ryr[10] = R45 * c.k54 * x2 * eq56;
        r.ryr[11] = (R)0;
    } else {
        r.ryr[5] = R4 * c.k56 * x2;
        r.ryr[9] = R4 * c.k52;
        r.ryr[10] = R4 * c.k54 * x2;
        r.ryr[11] = R5 * c.k65;
    }
    r.clch = ((s.flags >> (4 + j)) & 1u) == 0u ? c.kfClCh * x : c.kbClCh;
    R sub = r.lcc[0] + r.lcc[1] + r.lcc[2];
    sub = sub + r.inact;
#pragma unroll
    for (int k = 0; k < 12; ++k) sub = sub + r.ryr[k];
    sub = sub + r.clch;
    return sub;
}

// Table of the rates of subunit j other than the RyR rates, by the subunit's (LCC state, gate,
// ClCh) index: total = base + slope * CaSS.  base = the LCC state's V-dependent outgoing rates
// + the gate's rate + (ClCh open ? kbClCh : 0); slope = (Ca-dependent LCC inactivation: gamma0 a^k)
// + (ClCh closed ? kfClCh : 0).  Rebuilt by each CTA at the start of every global step (the
// V-dependent rates change per step); entry = state | gate << 4 | clch << 5.
constexpr int kRateTab = 64;

template <typename R>
__device__ __forceinline__ void build_rate_entry(float2 *tab, const SsaConsts<R> &c, const R *sv, int e) {
    const int st = e & 15, gate = (e >> 4) & 1, clch = (e >> 5) & 1;
    const uint32_t w = c.lcct[st];
    R base = sv[w & 0xFFu] + sv[(w >> 8) & 0xFFu] + sv[(w >> 16) & 0xFFu];
    base += gate ? sv[SV_INACT1] : sv[SV_INACT0];
    if (clch) base += c.kbClCh;
    R slope = ((w >> 24) < 3u && st >= 1) ? c.gam[(st - 1) & 7] : (R)0;
    if (!clch) slope += c.kfClCh;
    tab[e] = make_float2((float)base, (float)slope);
}

// Byte j of the result: subunit j's rate-table index (LCC state | gate << 4 | ClCh << 5).
__device__ __forceinline__ uint32_t rate_index_word(uint32_t lcc, uint32_t flags) {
    const uint32_t g = ((flags & 0xFu) * 0x00204081u) & 0x01010101u;         // gate bit j -> bit 8j
    const uint32_t k = (((flags >> 4) & 0xFu) * 0x00204081u) & 0x01010101u;  // ClCh bit j -> bit 8j
    return lcc | (g << 4) | (k << 5);
}

// FP32 total outgoing rate of subunit j (used only to draw the jump time and the subunit; the
// transition itself is drawn from the full rate list of subunit_rates): the table part plus the
// RyR rates regrouped.
template <typename R>
__device__ __forceinline__ R subunit_total_fast(const Cru<R> &s, int j, R x, const SsaConsts<R> &c,
                                                const float2 *tab, uint32_t iw) {
    const float2 tv = tab[(iw >> (8 * j)) & 0x3Fu];
    const R other = fmaf(tv.y, x, tv.x);
    const R R0 = (R)byte_s(s.ryr[0], j), R1 = (R)byte_s(s.ryr[1], j), R2 = (R)byte_s(s.ryr[2], j);
    const R R3 = (R)byte_s(s.ryr[3], j), R4 = (R)byte_s(s.ryr[4], j), R5 = (R)byte_s(s.ryr[5], j);
    const R x2 = x * x;
    R ryr = x2 * (R0 * c.k12 + R1 * c.k2325) + R1 * c.k21;
    if (x > (R)3.685e-2)
        ryr += (R2 + R3) * __fdividef((float)(c.k45k34 * x2 + c.k32k43), (float)(c.k34 * x2 + c.k43));
    else
        ryr += x2 * R2 * c.k34 + R3 * c.k4543 + R2 * c.k32;
    if (x > (R)1.15e-4)
        ryr += (R4 + R5) * __fdividef((float)(c.k65 * (c.k52 + c.k54 * x2)), (float)(c.k56 * x2 + c.k65));
    else
        ryr += x2 * R4 * c.k5654 + R4 * c.k52 + R5 * c.k65;
    return other + ryr;
}

// sample_weights (common.hpp:49-59) with the draw already scaled: u = U * total.  In FP32 mode a
// scan that runs past the last positive weight (possible when rounding makes the partial sums fall
// short of u) is moved back to the last positive weight.
template <typename R, int N, bool GUARD>
__device__ __forceinline__ int scan_weights(const R *w, R u) {
    R cum = w[0];
    int idx = 0;
    bool go = cum < u;
#pragma unroll
    for (int i = 1; i < N; ++i) {
        if (go) {
            idx = i;
            cum += w[i];
            go = cum < u;
        }
    }
    if (GUARD) {
        int lp = 0;
#pragma unroll
        for (int i = 0; i < N; ++i)
            if (i <= idx && w[i] > (R)0) lp = i;
        idx = lp;
    }
    return idx;
}

// RyR transition table of sample_RyR (SSA.tpp:200-259): from state, to state (0-based).
__device__ __forceinline__ void ryr_move(int tr, int &from, int &to) {
    // transitions 0..11: 1->2, 2->3, 2->5, 3->4, 4->5, 5->6, 2->1, 3->2, 4->3, 5->2, 5->4, 6->5
    constexpr uint32_t F = 0u | (1u << 4) | (1u << 8) | (2u << 12) | (3u << 16) | (4u << 20) |
                           (1u << 24) | (2u << 28);
    constexpr uint32_t F2 = 3u | (4u << 4) | (4u << 8) | (5u << 12);
    constexpr uint32_t T = 1u | (2u << 4) | (4u << 8) | (3u << 12) | (4u << 16) | (5u << 20) |
                           (0u << 24) | (1u << 28);
    constexpr uint32_t T2 = 2u | (1u << 4) | (3u << 8) | (4u << 12);
    if (tr < 8) {
        from = (int)((F >> (4 * tr)) & 0xFu);
        to = (int)((T >> (4 * tr)) & 0xFu);
    } else {
        from = (int)((F2 >> (4 * (tr - 8))) & 0xFu);
        to = (int)((T2 >> (4 * (tr - 8))) & 0xFu);
    }
}

// sample_RyR56 / sample_RyR34 (SSA.tpp:59-84) on the byte pair (a, b) of subunit j: n = a + b
// Bernoulli(p) draws (sample_binomial, common.hpp:37-47) from draw index kr on.
template <typename R>
__device__ __forceinline__ void resplit_pair(uint32_t &a, uint32_t &b, int j, R p, Stream &rng,
                                             uint32_t &kr) {
    const int n = byte_s(a, j) + byte_s(b, j);
    if (n > 0) {
        int X = 0;
        for (int i = 0; i < n; ++i)
            if (rng.uniform<R>(kr++) < p) ++X;
        a = byte_set(a, j, X);
        b = byte_set(b, j, n - X);
    } else {
        a = byte_set(a, j, 0);
        b = byte_set(b, j, 0);
    }
}


// One CRU over one global step: SSA_single_CRU (SSA.tpp:286-310) with the reference's draw order.
// The jump draw comes first; then update_CaSS's binomial re-splits (sample_RyR56/34), then the
// subunit and transition draws.  The transition is chosen from the rates of the start of the
// iteration (as the reference's stored rate arrays are) and applied after the Ca update, so the
// code reorders independent work but not values: re-split draws use indices k+1..k+D and the
// selection draws k+D+1.. exactly as the reference's sequential urand() calls would.
//
// SsaLane holds the loop state of one CRU's step so that a lane can run one iteration at a time
// (the engine's SSA warps interleave CRUs: a lane whose CRU has finished its step takes the next
// CRU while lanes with pending events continue).

// Threshold crossing of update_CaSS (SSA.tpp:87-99) by subunit j from x to x_new: 1 when CaSS
// falls through 1.15e-4 (re-split of RyR states 5/6), else 2 when it falls through 3.685e-2
// (states 3/4), else 0.  A positive count of the pair adds its draws to D.
template <typename R>
__device__ __forceinline__ int crossing(const Cru<R> &s, int j, R x, R x_new, uint32_t &D) {
    if (x > (R)1.15e-4 && x_new <= (R)1.15e-4) {
        const int n = byte_s(s.ryr[4], j) + byte_s(s.ryr[5], j);
        if (n > 0) D += (uint32_t)n;
        return 1;
    }
    if (x > (R)0.03685 && x_new <= (R)0.03685) {
        const int n = byte_s(s.ryr[2], j) + byte_s(s.ryr[3], j);
        if (n > 0) D += (uint32_t)n;
        return 2;
    }
    return 0;
}

// Event selection (sample_weights over subunits, sample_new_state) from the rates of the start of
// the iteration with draws kk, kk+1, kk+2: act 1 LCC, 2 inactivation toggle, 3 RyR, 4 ClCh
// toggle; aj the subunit, atr the transition.
template <typename R, bool EXACT>
__device__ __forceinline__ void select_transition(const Rates<R> &r, R subr, Stream &rng, uint32_t &kk, int &act,
                                                  int &atr);
template <typename R, bool EXACT>
__device__ __forceinline__ void select_event(const Cru<R> &s, const SsaConsts<R> &c, const R *sv, const R (&sub)[4],
                                             R total, Stream &rng, uint32_t &kk, int &act, int &aj, int &atr) {
    const R us = rng.uniform<R>(kk++) * total;
    aj = scan_weights<R, 4, !EXACT>(sub, us);
    Rates<R> r;
    const R sr = subunit_rates<R>(s, aj, pick4(s.cass, aj), c, sv, r);
    select_transition<R, EXACT>(r, EXACT ? pick4(sub, aj) : sr, rng, kk, act, atr);
}

// sample_new_state's choice within subunit aj (SSA.tpp:262-283) from its rates r and total subr,
// with draws kk, kk+1: act 1 LCC, 2 inactivation toggle, 3 RyR, 4 ClCh toggle; atr the transition.
template <typename R, bool EXACT>
__device__ __forceinline__ void select_transition(const Rates<R> &r, R subr, Stream &rng, uint32_t &kk, int &act,
                                                  int &atr) {
    const R sum_lcc = r.lcc[0] + r.lcc[1] + r.lcc[2];
    R sum_ryr;
    if (EXACT) {
        sum_ryr = subr - (sum_lcc + r.inact + r.clch);
    } else {
        sum_ryr = (R)0;
#pragma unroll
        for (int q = 0; q < 12; ++q) sum_ryr += r.ryr[q];
    }
    const R u = rng.uniform<R>(kk++) * subr;
    if (u < sum_lcc) {
        act = 1;
        atr = scan_weights<R, 3, !EXACT>(r.lcc, rng.uniform<R>(kk++) * sum_lcc);
    } else if (u < (sum_lcc + r.inact)) {
        act = 2;
    } else if (u < (sum_lcc + r.inact + sum_ryr)) {
        act = 3;
        atr = scan_weights<R, 12, !EXACT>(r.ryr, rng.uniform<R>(kk++) * sum_ryr);
    } else {
        act = 4;
    }
}

// update_CaSS's second pass: binomial re-splits (sample_RyR56/34, SSA.tpp:59-84) of the subunits
// that crossed a threshold, with draws k+1 .. k+D; s.cass still holds the values before the update.
template <typename R>
__device__ __forceinline__ void resplit_crossed(Cru<R> &s, const SsaConsts<R> &c, const int (&kind)[4], Stream &rng,
                                                uint32_t k) {
    uint32_t kr = k + 1u;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        if (kind[j] == 0) continue;
        const R x = s.cass[j];
        if (kind[j] == 1)
            resplit_pair<R>(s.ryr[4], s.ryr[5], j, c.k65 / (c.k65 + c.k56 * (x * x)), rng, kr);
        else
            resplit_pair<R>(s.ryr[2], s.ryr[3], j, c.k43 / (c.k43 + c.k34 * (x * x)), rng, kr);
    }
}

// Element i of a 4-element register array set to v (predicated moves, no local memory).
template <typename T>
__device__ __forceinline__ void set4(T (&a)[4], int i, T v) {
    a[0] = i == 0 ? v : a[0];
    a[1] = i == 1 ? v : a[1];
    a[2] = i == 2 ? v : a[2];
    a[3] = i == 3 ? v : a[3];
}

// The transition (sample_new_state, SSA.tpp:262-283) applied to the updated state, with the JLCC
// and Jrel updates of sample_LCC and sample_RyR.  Works on subunit aj directly: byte fields by a
// shift of 8*aj, a RyR move as a per-byte modular addition (__vadd4) of +1 and -1 in byte aj of
// the two state planes.  Counts are signed bytes and may go below zero (a lumped 3/4 or 5/6 rate
// moves a RyR out of a state whose own count is 0, as in the reference), so the planes must not
// carry or borrow between subunits.
template <typename R>
__device__ __forceinline__ void apply_event(Cru<R> &s, const SsaConsts<R> &c, const R *sv, int act, int aj, int atr,
                                            R (&jrel)[4]) {
    const uint32_t sh = 8u * (uint32_t)aj;
    if (act == 1) {
        const int from = (int)((s.lcc >> sh) & 0xFFu);
        if (from >= 1 && from <= 12) {
            const int to = (int)((c.lccn[from] >> (4 * atr)) & 0xFu);
            s.lcc = (s.lcc & ~(0xFFu << sh)) | ((uint32_t)to << sh);
            const bool inact1 = ((s.flags >> aj) & 1u) != 0u;
            if ((from == 5 && to == 6) || (from == 11 && to == 12))
                set4(s.jlcc, aj, inact1 ? sv[SV_JMUL] * (c.Cao_scaled - sv[SV_JEXP] * pick4(s.cass, aj)) : (R)0);
            else if (from == 6 || from == 12)
                set4(s.jlcc, aj, (R)0);
        }
    } else if (act == 2) {
        s.flags ^= (1u << aj);
        const int st = (int)((s.lcc >> sh) & 0xFFu);
        if (((s.flags >> aj) & 1u) == 0u)
            set4(s.jlcc, aj, (R)0);
        else if (st == 6 || st == 12)
            set4(s.jlcc, aj, sv[SV_JMUL] * (c.Cao_scaled - sv[SV_JEXP] * pick4(s.cass, aj)));
    } else if (act == 3) {
        int from, to;
        ryr_move(atr, from, to);
        const uint32_t up = 1u << sh, down = 0xFFu << sh;  // +1 and -1 (mod 256) in byte aj
#pragma unroll
        for (int q = 0; q < 6; ++q) s.ryr[q] = __vadd4(s.ryr[q], q == to ? up : (q == from ? down : 0u));
        const R open = (R)(byte_s(s.ryr[2], aj) + byte_s(s.ryr[3], aj));
        set4(jrel, aj, c.rRyR * open * (s.cajsr - pick4(s.cass, aj)));
    } else {
        s.flags ^= (1u << (4 + aj));
    }
}

// What one iteration of the event loop did: its sub-step length (the jump time, or the rest of the
// global step for the last one) and the event chosen after it (act 0: none; else act, subunit aj
// and transition atr as select_event returns them).  Read by the pathwise adjoint (gw_adjoint.cu).
template <typename R>
struct IterInfo {
    R h;
    int act, aj, atr;
};

// ------------------------------------------------------------------------------------------
// FP32 screen of the FP64 lane's jump decision (SsaLane::surely_last).
// ------------------------------------------------------------------------------------------
// FP64 lanes whose iteration the screen declined wait until this many lanes of their warp do (or
// the warp has no CRUs left to take), then run the FP64 iteration together.
constexpr int kDefer = 8;

// Float copies of the rate constants the screen uses; SK_OK is 1 when all of them are
// non-negative (the error bound assumes sums of non-negative factors in the reciprocals), else the
// screen declines every iteration.
enum ScreenConst {
    SK_K12, SK_K21, SK_K23, SK_K32, SK_K34, SK_K43, SK_K45, SK_K54, SK_K56, SK_K65, SK_K25, SK_K52,
    SK_KFCLCH, SK_KBCLCH, SK_GAM, SK_OK = SK_GAM + 5, SK_COUNT
};
__device__ __forceinline__ void load_screen_consts(float *sk, const CellStatic &s) {
    const gw_params &p = s.p;
    sk[SK_K12] = (float)p.k12; sk[SK_K21] = (float)p.k21; sk[SK_K23] = (float)p.k23; sk[SK_K32] = (float)p.k32;
    sk[SK_K34] = (float)p.k34; sk[SK_K43] = (float)p.k43; sk[SK_K45] = (float)p.k45; sk[SK_K54] = (float)p.k54;
    sk[SK_K56] = (float)p.k56; sk[SK_K65] = (float)p.k65; sk[SK_K25] = (float)p.k25; sk[SK_K52] = (float)p.k52;
    sk[SK_KFCLCH] = (float)p.kfClCh; sk[SK_KBCLCH] = (float)p.kbClCh;
    sk[SK_GAM + 0] = (float)s.gamma0; sk[SK_GAM + 1] = (float)s.gamma0a; sk[SK_GAM + 2] = (float)s.gamma0a2;
    sk[SK_GAM + 3] = (float)s.gamma0a3; sk[SK_GAM + 4] = (float)s.gamma0a4;
    bool ok = true;
    for (int i = 0; i < SK_OK; ++i) ok = ok && sk[i] >= 0.f;
    sk[SK_OK] = ok ? 1.f : 0.f;
}

// f = d with its significand truncated to 24 bits (|f - d| <= 2^-23 |d|), by integer operations
// (an FP64 -> FP32 conversion would take the FP64 pipe); false unless d is zero or in the normal
// FP32 range.
__device__ __forceinline__ bool f32_trunc(double d, float &f) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(d);
    const uint32_t hi = (uint32_t)(b >> 32), lo = (uint32_t)b;
    const uint32_t e = (hi >> 20) & 0x7FFu;
    const bool zero = (b << 1) == 0ull;
    f = zero ? 0.f : __uint_as_float((hi & 0x80000000u) | ((e - 896u) << 23) | ((hi & 0xFFFFFu) << 3) | (lo >> 29));
    return zero || (e > 896u && e < 1151u);
}

// Signed byte j of a RyR plane word as a float: the byte, biased by 128, becomes the low byte of
// the bit pattern of 2^23 + 128 + n.
__device__ __forceinline__ float count_f(uint32_t w, int j) {
    return __uint_as_float(__byte_perm(w ^ 0x80808080u, 0x4B000000u, (uint32_t)j | 0x7540u)) - 8388736.f;
}

// The 17 rates of subunit j as subunit_rates computes them (same regimes and formulas, FP32),
// added to T and their magnitudes to A.  x: CaSS of the subunit (FP32), xb: its FP64 bits.
template <typename R>
__device__ __forceinline__ void screen_subunit(const Cru<R> &s, int j, float x, long long xb, const SsaConsts<R> &c,
                                               const float *sk, const float *svf, float &T, float &A) {
    const int st = byte_u(s.lcc, j);
    const uint32_t w = c.lcct[st & 15];
    float l0 = svf[w & 0xFFu], l1 = svf[(w >> 8) & 0xFFu], l2 = svf[(w >> 16) & 0xFFu];
    const int kin = (int)(w >> 24);
    if (kin < 3) {
        const float gx = sk[SK_GAM + st - 1] * x;
        if (kin == 1) l1 = gx; else l2 = gx;
    }
    const float inact = ((s.flags >> j) & 1u) == 0u ? svf[SV_INACT0] : svf[SV_INACT1];
    const float clch = ((s.flags >> (4 + j)) & 1u) == 0u ? sk[SK_KFCLCH] * x : sk[SK_KBCLCH];
    const float R0 = count_f(s.ryr[0], j), R1 = count_f(s.ryr[1], j), R2 = count_f(s.ryr[2], j);
    const float R3 = count_f(s.ryr[3], j), R4 = count_f(s.ryr[4], j), R5 = count_f(s.ryr[5], j);
    const float R23 = R2 + R3, R45 = R4 + R5;  // exact: small integers
    const float x2 = x * x;
    float r[12];
    r[0] = R0 * sk[SK_K12] * x2;
    r[1] = R1 * sk[SK_K23] * x2;
    r[2] = R1 * sk[SK_K25] * x2;
    r[6] = R1 * sk[SK_K21];
    // x > 3.685e-2 and x > 1.15e-4 of the FP64 code, on the bit patterns
    if (xb > __double_as_longlong(3.685e-2)) {
        const float tau34 = __fdividef(1.f, sk[SK_K34] * x2 + sk[SK_K43]);
        r[3] = 0.f;
        r[4] = R23 * sk[SK_K45] * sk[SK_K34] * x2 * tau34;
        r[7] = R23 * sk[SK_K32] * sk[SK_K43] * tau34;
        r[8] = 0.f;
    } else {
        r[3] = R2 * sk[SK_K34] * x2;
        r[4] = R3 * sk[SK_K45];
        r[7] = R2 * sk[SK_K32];
        r[8] = R3 * sk[SK_K43];
    }
    if (xb > __double_as_longlong(1.15e-4)) {
        const float eq56 = __fdividef(sk[SK_K65], sk[SK_K56] * x2 + sk[SK_K65]);
        r[5] = 0.f;
        r[9] = R45 * sk[SK_K52] * eq56;
        r[10] = R45 * sk[SK_K54] * x2 * eq56;
        r[11] = 0.f;
    } else {
        r[5] = R4 * sk[SK_K56] * x2;
        r[9] = R4 * sk[SK_K52];
        r[10] = R4 * sk[SK_K54] * x2;
        r[11] = R5 * sk[SK_K65];
    }
    T += ((l0 + l1) + (l2 + inact)) + clch;
    A += ((fabsf(l0) + fabsf(l1)) + (fabsf(l2) + fabsf(inact))) + fabsf(clch);
#pragma unroll
    for (int q = 0; q < 12; ++q) {
        T += r[q];
        A += fabsf(r[q]);
    }
}

template <typename R, bool EXACT>
struct SsaLane {
    R t;          // time reached within the global step
    uint32_t k;   // next draw index
    int ev;       // events so far in this step
    R jrel[4];    // Jrel, updated at the start of the step and at RyR transitions (SSA.tpp:10-33)
    R jxfer_sum;  // sum over subunits of Jxfer of the last update_fluxes
    R jtr;        // Jtr of the last update_fluxes

    __device__ __forceinline__ void begin(const Cru<R> &s, const SsaConsts<R> &c) {
        t = (R)0;
        k = 0;
        ev = 0;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const R open = (R)(byte_s(s.ryr[2], j) + byte_s(s.ryr[3], j));
            jrel[j] = c.rRyR * open * (s.cajsr - s.cass[j]);
        }
    }

    // update_fluxes (SSA.tpp:37-45): Jtr (kept in jtr), Jiss and Jxfer of the CRU's current state.
    __device__ __forceinline__ void fluxes(const Cru<R> &s, const SsaConsts<R> &c, const R *sv, R (&jxfer)[4],
                                           R (&jiss)[4]) {
        const R Cai = sv[SV_CAI], CaNSR = sv[SV_CANSR];
        const R Cai_lo = EXACT ? (R)0 : sv[SV_CAI_LO], CaNSR_lo = EXACT ? (R)0 : sv[SV_CANSR_LO];
        if (EXACT) {
            jtr = c.rtr * (CaNSR - s.cajsr);
        } else {
            jtr = c.rtr * ((CaNSR - s.cajsr) + (CaNSR_lo - (R)s.cajsr_lo));
        }
        jiss[0] = c.riss * (s.cass[1] + s.cass[3] - (R)2 * s.cass[0]);
        jiss[1] = c.riss * (s.cass[2] + s.cass[0] - (R)2 * s.cass[1]);
        jiss[2] = c.riss * (s.cass[3] + s.cass[1] - (R)2 * s.cass[2]);
        jiss[3] = c.riss * (s.cass[0] + s.cass[2] - (R)2 * s.cass[3]);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            if (EXACT)
                jxfer[j] = c.rxfer * (s.cass[j] - Cai);
            else
                jxfer[j] = c.rxfer * ((s.cass[j] - Cai) - Cai_lo);
        }
    }

    // One iteration of the event loop; true when the CRU's step is complete (the jump passed the
    // end of the step, or the event cap was exceeded, which sets err).
    __device__ __forceinline__ bool iterate(Cru<R> &s, const SsaConsts<R> &c, const R *sv, const float2 *tab,
                                            Stream &rng, R dt, int cap, int &err, IterInfo<R> *info = nullptr) {
        R jxfer[4], jiss[4];
        fluxes(s, c, sv, jxfer, jiss);
        // update_rates (SSA.tpp:48-56): only the subunit totals are kept here.
        R sub[4];
        const uint32_t iw = EXACT ? 0u : rate_index_word(s.lcc, s.flags);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            if (EXACT) {
                Rates<R> r;
                sub[j] = subunit_rates<R>(s, j, s.cass[j], c, sv, r);
            } else {
                sub[j] = subunit_total_fast<R>(s, j, s.cass[j], c, tab, iw);
            }
        }
        const R total = sub[0] + sub[1] + sub[2] + sub[3];
        const R u0 = rng.uniform<R>(k);
        R jump;
        if (EXACT)
            jump = -log(u0) / total;
        else
            jump = __fdividef(-logf((float)u0), (float)total);
        const bool last = !(t + jump < dt);
        const R h = last ? (dt - t) : jump;
        return advance(s, c, sv, rng, h, last, jump, sub, total, jxfer, jiss, cap, err, info);
    }

    // The step's last iteration of a CRU whose jump is known to pass the end of the step (see
    // surely_last): iterate() without the rate evaluation and the jump draw, which such an
    // iteration does not use.  Same expressions in the same order, so the same results.
    __device__ __forceinline__ void finish(Cru<R> &s, const SsaConsts<R> &c, const R *sv, Stream &rng, R dt,
                                           IterInfo<R> *info = nullptr) {
        R jxfer[4], jiss[4];
        fluxes(s, c, sv, jxfer, jiss);
        const R none[4] = {(R)0, (R)0, (R)0, (R)0};
        int err = 0;
        advance(s, c, sv, rng, dt - t, true, (R)0, none, (R)0, jxfer, jiss, 0, err, info);
    }

    // update_CaSS (SSA.tpp:87-99), first pass, for subunit j: its new CaSS (tmp_j) and threshold
    // crossing (kind_j; a positive count of the re-split pair adds its draws to D).
    __device__ __forceinline__ void cass_update(const Cru<R> &s, const SsaConsts<R> &c, int j, R h,
                                                const R (&jxfer)[4], const R (&jiss)[4], R &tmp_j, int &kind_j,
                                                uint32_t &D) const {
        // (pick4: j may be a lane's own subunit, and a register array indexed by a value known only
        // at run time would go to local memory)
        const R x = pick4(s.cass, j);
        R beta;
        if (EXACT) {
            beta = (R)1.0 / ((R)1 + (c.BSR_const / ((c.KBSR + x) * (c.KBSR + x))) +
                             (c.BSL_const / ((c.KBSL + x) * (c.KBSL + x))));
        } else {
            const R u = (c.KBSR + x) * (c.KBSR + x), v = (c.KBSL + x) * (c.KBSL + x);
            const R uv = u * v;
            beta = __fdividef((float)uv, (float)(uv + c.BSR_const * v + c.BSL_const * u));
        }
        const R d = h * (pick4(s.jlcc, j) + pick4(jrel, j) - pick4(jxfer, j) + pick4(jiss, j)) * beta;
        tmp_j = x + d;
        kind_j = crossing<R>(s, j, x, tmp_j, D);
    }

    // The iteration once its sub-step h is known: update_CaSS with its re-splits, the event choice
    // (not on the last iteration), update_CaJSR and the transition.
    __device__ __forceinline__ bool advance(Cru<R> &s, const SsaConsts<R> &c, const R *sv, Stream &rng, R h,
                                            bool last, R jump, const R (&sub)[4], R total, const R (&jxfer)[4],
                                            const R (&jiss)[4], int cap, int &err, IterInfo<R> *info) {
        R tmp[4];
        int kind[4];
        uint32_t D = 0;
#pragma unroll
        for (int j = 0; j < 4; ++j) cass_update(s, c, j, h, jxfer, jiss, tmp[j], kind[j], D);
        // Event selection from the rates of the start of this iteration, draws k+D+1, k+D+2, k+D+3.
        uint32_t kk = k + 1u + D;
        int act = 0, aj = 0, atr = 0;
        if (!last) {
            t += jump;
            select_event<R, EXACT>(s, c, sv, sub, total, rng, kk, act, aj, atr);
        }
        return conclude(s, c, sv, rng, h, last, tmp, kind, D, kk, act, aj, atr, jxfer, cap, err, info);
    }

    // The iteration's end: update_CaSS's second pass and commit, update_CaJSR (SSA.hpp:68-71), the
    // transition, and the loop state.
    __device__ __forceinline__ bool conclude(Cru<R> &s, const SsaConsts<R> &c, const R *sv, Stream &rng, R h,
                                             bool last, const R (&tmp)[4], const int (&kind)[4], uint32_t D,
                                             uint32_t kk, int act, int aj, int atr, const R (&jxfer)[4], int cap,
                                             int &err, IterInfo<R> *info) {
        if (D > 0 || kind[0] || kind[1] || kind[2] || kind[3]) resplit_crossed<R>(s, c, kind, rng, k);
#pragma unroll
        for (int j = 0; j < 4; ++j) s.cass[j] = tmp[j];
        {
            const R x = s.cajsr;
            R beta;
            if (EXACT)
                beta = (R)1.0 / ((R)1 + c.CSQN_const / ((c.KCSQN + x) * (c.KCSQN + x)));
            else {
                const R u = (c.KCSQN + x) * (c.KCSQN + x);
                beta = __fdividef((float)u, (float)(u + c.CSQN_const));
            }
            const R d = h * beta * (jtr - c.VSS_VJSR * (jrel[0] + jrel[1] + jrel[2] + jrel[3]));
            if (EXACT) {
                s.cajsr += d;
            } else {
                // Fast2Sum into (hi, lo): near rest the per-step JSR increment is below half an
                // ulp of CaJSR in FP32, and would otherwise be lost.
                const float hi = (float)s.cajsr;
                const float y = (float)d + s.cajsr_lo;
                const float sum = hi + y;
                const float err_ = y - (sum - hi);
                s.cajsr = (R)sum;
                s.cajsr_lo = err_;
            }
        }
        // Apply the transition to the updated state.
        if (act != 0) apply_event<R>(s, c, sv, act, aj, atr, jrel);
        if (info) {
            info->h = h;
            info->act = act;
            info->aj = aj;
            info->atr = atr;
        }
        jxfer_sum = jxfer[0] + jxfer[1] + jxfer[2] + jxfer[3];
        k = kk;
        if (last) return true;
        if (++ev > cap) {
            err = 1;
            return true;
        }
        return false;
    }

    // iterate() by the four lanes of a group (lanes 4g .. 4g+3 of the warp, every one holding the
    // same CRU and lane state; EXACT, R = double): lane j = lane & 3 evaluates the 17 rates and the
    // CaSS update of subunit j, the group exchanges them by shuffles, and the rest runs on the four
    // lanes alike.  Same expressions in the same order as iterate(), hence the same results on every
    // lane; an FP64 warp instruction costs the same whatever its active lanes, so the iteration takes
    // about a third of the FP64 instructions of one lane's.  The four lanes must call it together.
    __device__ __forceinline__ bool iterate_group(Cru<R> &s, const SsaConsts<R> &c, const R *sv, Stream &rng, R dt,
                                                  int cap, int &err) {
        static_assert(sizeof(R) == 8 && EXACT, "the group iteration is for the FP64 lane");
        const int lane = (int)(threadIdx.x & 31u), j = lane & 3, base = lane & ~3;
        const unsigned gm = 0xFu << base;
        R jxfer[4], jiss[4];
        fluxes(s, c, sv, jxfer, jiss);
        Rates<R> rj;
        const R sj = subunit_rates<R>(s, j, pick4(s.cass, j), c, sv, rj);
        R sub[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) sub[q] = __shfl_sync(gm, sj, base + q);
        const R total = sub[0] + sub[1] + sub[2] + sub[3];
        const R u0 = rng.uniform<R>(k);
        const R jump = -log(u0) / total;
        const bool last = !(t + jump < dt);
        const R h = last ? (dt - t) : jump;
        R tj;
        int kj;
        uint32_t Dj = 0;
        cass_update(s, c, j, h, jxfer, jiss, tj, kj, Dj);
        R tmp[4];
        int kind[4];
        uint32_t D = 0;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            tmp[q] = __shfl_sync(gm, tj, base + q);
            kind[q] = __shfl_sync(gm, kj, base + q);
            D += __shfl_sync(gm, Dj, base + q);
        }
        uint32_t kk = k + 1u + D;
        int act = 0, aj = 0, atr = 0;
        if (!last) {
            t += jump;
            // select_event with the drawn subunit's rates from its lane
            const R us = rng.uniform<R>(kk++) * total;
            aj = scan_weights<R, 4, false>(sub, us);
            const int src = base + aj;
            Rates<R> r;
#pragma unroll
            for (int q = 0; q < 3; ++q) r.lcc[q] = __shfl_sync(gm, rj.lcc[q], src);
            r.inact = __shfl_sync(gm, rj.inact, src);
#pragma unroll
            for (int q = 0; q < 12; ++q) r.ryr[q] = __shfl_sync(gm, rj.ryr[q], src);
            r.clch = __shfl_sync(gm, rj.clch, src);
            select_transition<R, true>(r, pick4(sub, aj), rng, kk, act, atr);
        }
        return conclude(s, c, sv, rng, h, last, tmp, kind, D, kk, act, aj, atr, jxfer, cap, err, nullptr);
    }

    // FP32 screen of the next FP64 iteration (EXACT, R = double): true only if that iteration is
    // certainly the step's last, i.e. its jump -log(u0) / total passes dt - t.  An FP64 iteration
    // spends most of its FP64 instructions on the 68 rates and the log and division of the jump
    // time, which the last iteration does not otherwise use; an FP64 instruction takes a warp
    // scheduler's FP64 pipe for ~64 cycles, an FP32 one for one or two.  The screen evaluates the
    // rates in FP32 from CaSS truncated to FP32 and float copies of the constants (sk) and the
    // step's SSA values (svf):
    //   T = their sum, A = the sum of their magnitudes.  Every rate is a product of at most five
    //   factors with at most one reciprocal, so it is within ~2e-6 of the FP64 rate relative to
    //   itself; the sum adds at most 67 roundings of 2^-24 of A: |T - total| <= 7e-6 A.  The
    //   regime tests (CaSS above 3.685e-2 and 1.15e-4) compare the FP64 bit patterns as integers,
    //   which orders non-negative doubles exactly as the FP64 compare does, so both sides take the
    //   same branches (a NaN fails the screen through T).
    //   u0 = max(w >> 11, 1) 2^-53 <= ((w >> 40) + 1) 2^-24 = u_hi, exact in FP32.
    // The FP64 iteration finds the jump past the end when -log(u0) >= total (dt - t) (1 + 1e-5)
    // and total > 0: then jump = -log(u0) / total, both rounded to within a few ulp, exceeds the
    // exact dt - t, and t + jump rounds to at least dt.  The screen asks for
    //   T - 1e-4 A > 0  and  u_hi <= 0.9999 exp(-(T + 1e-4 A) h (1 + 2e-5)),
    // h = dt - t truncated to FP32, with __expf's relative error (~4e-6 for arguments below 88)
    // inside the 1e-4 margin.  It declines (and the FP64 iteration decides) in the few cases within
    // those margins, and on every iteration that has an event.
    __device__ __forceinline__ bool surely_last(const Cru<R> &s, const SsaConsts<R> &c, const float *sk,
                                                const float *svf, Stream &rng, R dt) {
        static_assert(sizeof(R) == 8 && EXACT, "the screen is for the FP64 lane");
        float T = 0.f, A = 0.f;
        bool ok = true;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const long long xb = __double_as_longlong(s.cass[j]);
            float x;
            ok &= f32_trunc(s.cass[j], x);
            screen_subunit(s, j, x, xb, c, sk, svf, T, A);
        }
        uint32_t hi, lo;
        rng.words(k, hi, lo);
        const float u_hi = __uint2float_rn((hi >> 8) + 1u) * 0x1p-24f;
        float h;
        ok &= f32_trunc(dt - t, h);
        const float Thi = fmaf(1e-4f, A, T), Tlo = fmaf(-1e-4f, A, T);
        const float X = Thi * h * 1.00002f;
        return ok && sk[SK_OK] != 0.f && Tlo > 0.f && u_hi <= __expf(-X) * 0.9999f;
    }
};

// ------------------------------------------------------------------------------------------
// FP32 lane on subunit pairs.  The iteration of the generic lane (same formulas, same draws) with
// subunits (0,1) and (2,3) held as float2 pairs for the packed FP32x2 instructions of sm_100 and
// later (FFMA2, FADD2, FMUL2: each half rounds as the scalar instruction).  RyR counts become
// floats by a byte permute into the bit pattern of 2^23 + 128 + n and one packed subtraction.
// Sums over the four subunits are taken as (0+2) + (1+3).
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }
// x / y as x * rcp.approx(y), the arithmetic of __fdividef without its guard for |y| > 2^126 (the
// divisors here are rate sums and buffer terms far below that)
__device__ __forceinline__ float rcp_approx(float y) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(y));
    return r;
}
__device__ __forceinline__ float2 div2(float2 x, float2 y) {
    return __fmul2_rn(x, make_float2(rcp_approx(y.x), rcp_approx(y.y)));
}

// Signed byte counts of subunits 2p and 2p+1 from a RyR plane word whose bytes carry a +0x80 bias
// (w ^ 0x80808080): float(0x4B0000bb) = 2^23 + bb, less 2^23 + 128.
__device__ __forceinline__ float2 counts2(uint32_t wb, int p, float2 bias) {
    const float a = __uint_as_float(__byte_perm(wb, 0x4B000000u, (uint32_t)(2 * p) | 0x7540u));
    const float b = __uint_as_float(__byte_perm(wb, 0x4B000000u, (uint32_t)(2 * p + 1) | 0x7540u));
    return add2(make_float2(a, b), bias);
}

// The 12 RyR rates of subunit j (update_RyR_rates, GW_utils.tpp:222-255) in FP32, with the two
// divisions of the lumped regimes as reciprocal estimates (rcp_approx), as in the subunit totals.
__device__ __forceinline__ void ryr_rates_f32(const Cru<float> &s, int j, float x, const SsaConsts<float> &c,
                                              float (&r)[12]) {
    const float R0 = (float)byte_s(s.ryr[0], j), R1 = (float)byte_s(s.ryr[1], j), R2 = (float)byte_s(s.ryr[2], j);
    const float R3 = (float)byte_s(s.ryr[3], j), R4 = (float)byte_s(s.ryr[4], j), R5 = (float)byte_s(s.ryr[5], j);
    const float R23 = (float)(byte_s(s.ryr[2], j) + byte_s(s.ryr[3], j));
    const float R45 = (float)(byte_s(s.ryr[4], j) + byte_s(s.ryr[5], j));
    const float x2 = x * x;
    r[0] = R0 * c.k12 * x2;
    r[1] = R1 * c.k23 * x2;
    r[2] = R1 * c.k25 * x2;
    r[6] = R1 * c.k21;
    if (x > 3.685e-2f) {
        const float tau34 = rcp_approx(c.k34 * x2 + c.k43);
        r[3] = 0.f;
        r[4] = R23 * c.k45 * c.k34 * x2 * tau34;
        r[7] = R23 * c.k32 * c.k43 * tau34;
        r[8] = 0.f;
    } else {
        r[3] = R2 * c.k34 * x2;
        r[4] = R3 * c.k45;
        r[7] = R2 * c.k32;
        r[8] = R3 * c.k43;
    }
    if (x > 1.15e-4f) {
        const float eq56 = c.k65 * rcp_approx(c.k56 * x2 + c.k65);
        r[5] = 0.f;
        r[9] = R45 * c.k52 * eq56;
        r[10] = R45 * c.k54 * x2 * eq56;
        r[11] = 0.f;
    } else {
        r[5] = R4 * c.k56 * x2;
        r[9] = R4 * c.k52;
        r[10] = R4 * c.k54 * x2;
        r[11] = R5 * c.k65;
    }
}

// FP32 event selection: select_event's draws and decisions, with the subunit's RyR total taken
// from the iteration's packed total computation (ryr_sub) and the 12 individual RyR rates formed
// only when the RyR class is drawn (at rest most events are LCC and gate transitions).  The three
// draws are formed up front (Stream::u24x3); a selection uses two or three of them, as
// select_event's sequential draws would.
__device__ __forceinline__ void select_event_f32(const Cru<float> &s, const SsaConsts<float> &c, const float *sv,
                                                 const float (&sub)[4], const float (&ryr_sub)[4], float total,
                                                 Stream &rng, uint32_t &kk, int &act, int &aj, int &atr) {
    float ua, ub, uc;
    rng.u24x3(kk, ua, ub, uc);
    const float us = ua * total;
    aj = scan_weights<float, 4, true>(sub, us);
    const float x = pick4(s.cass, aj);
    // update_LCC_rates, update_LCC_inactivation_rates, update_ClCh_rates of subunit aj
    const int st = byte_u(s.lcc, aj);
    const uint32_t w = c.lcct[st & 15];
    float lcc[3] = {sv[w & 0xFFu], sv[(w >> 8) & 0xFFu], sv[(w >> 16) & 0xFFu]};
    const int kin = (int)(w >> 24);
    if (kin < 3) {
        const float gx = c.gam[st - 1] * x;
        if (kin == 1) lcc[1] = gx; else lcc[2] = gx;
    }
    const float inact = ((s.flags >> aj) & 1u) == 0u ? sv[SV_INACT0] : sv[SV_INACT1];
    const float clch = ((s.flags >> (4 + aj)) & 1u) == 0u ? c.kfClCh * x : c.kbClCh;
    const float sum_lcc = lcc[0] + lcc[1] + lcc[2];
    const float sum_ryr = pick4(ryr_sub, aj);
    const float subr = ((sum_lcc + inact) + sum_ryr) + clch;
    const float u = ub * subr;
    kk += 2u;
    if (u < sum_lcc) {
        act = 1;
        atr = scan_weights<float, 3, true>(lcc, uc * sum_lcc);
        kk += 1u;
    } else if (u < sum_lcc + inact) {
        act = 2;
    } else if (u < sum_lcc + inact + sum_ryr) {
        act = 3;
        float r[12];
        ryr_rates_f32(s, aj, x, c, r);
        // the rates' sum in three groups of four (independent chains), then the sequential scan
        const float g0 = ((r[0] + r[1]) + r[2]) + r[3];
        const float g1 = ((r[4] + r[5]) + r[6]) + r[7];
        const float g2 = ((r[8] + r[9]) + r[10]) + r[11];
        atr = scan_weights<float, 12, true>(r, uc * ((g0 + g1) + g2));
        kk += 1u;
    } else {
        act = 4;
    }
}

template <>
struct SsaLane<float, false> {
    float t;
    uint32_t k;
    int ev;
    float jrel[4];
    float jxfer_sum;
    float jtr;

    __device__ __forceinline__ void begin(const Cru<float> &s, const SsaConsts<float> &c) {
        t = 0.f;
        k = 0;
        ev = 0;
        const float2 *K = c.pk;
        const uint32_t b2 = s.ryr[2] ^ 0x80808080u, b3 = s.ryr[3] ^ 0x80808080u;
        const float2 cj = make_float2(s.cajsr, s.cajsr);
#pragma unroll
        for (int p = 0; p < 2; ++p) {
            const float2 open = add2(counts2(b2, p, K[PK_BIAS]), counts2(b3, p, K[PK_BIAS]));
            const float2 x = make_float2(s.cass[2 * p], s.cass[2 * p + 1]);
            const float2 jr = mul2(mul2(K[PK_RRYR], open), add2(cj, neg2(x)));
            jrel[2 * p] = jr.x;
            jrel[2 * p + 1] = jr.y;
        }
    }

    __device__ __forceinline__ bool iterate(Cru<float> &s, const SsaConsts<float> &c, const float *sv,
                                            const float2 *tab, Stream &rng, float dt, int cap, int &err) {
        const float2 *K = c.pk;
        const float Cai = sv[SV_CAI], CaNSR = sv[SV_CANSR], Cai_lo = sv[SV_CAI_LO], CaNSR_lo = sv[SV_CANSR_LO];
        const float2 C[2] = {make_float2(s.cass[0], s.cass[1]), make_float2(s.cass[2], s.cass[3])};
        // update_fluxes (SSA.tpp:37-45)
        jtr = c.rtr * ((CaNSR - s.cajsr) + (CaNSR_lo - s.cajsr_lo));
        const float2 eo = add2(C[0], C[1]);  // (c0 + c2, c1 + c3)
        const float2 oe = make_float2(eo.y, eo.x);
        float2 jiss[2], jx[2];
        const float2 ncai = make_float2(-Cai, -Cai), ncailo = make_float2(-Cai_lo, -Cai_lo);
#pragma unroll
        for (int p = 0; p < 2; ++p) {
            jiss[p] = mul2(K[PK_RISS], fma2(K[PK_M2], C[p], oe));
            jx[p] = mul2(K[PK_RXFER], add2(add2(C[p], ncai), ncailo));
        }
        // subunit totals (the FP32 regrouping of subunit_total_fast)
        const uint32_t iw = rate_index_word(s.lcc, s.flags);
        const uint32_t b0 = s.ryr[0] ^ 0x80808080u, b1 = s.ryr[1] ^ 0x80808080u, b2 = s.ryr[2] ^ 0x80808080u;
        const uint32_t b3 = s.ryr[3] ^ 0x80808080u, b4 = s.ryr[4] ^ 0x80808080u, b5 = s.ryr[5] ^ 0x80808080u;
        float2 S[2], Y[2];  // subunit totals, and their RyR parts
#pragma unroll
        for (int p = 0; p < 2; ++p) {
            const float2 X = C[p];
            const float2 X2 = mul2(X, X);
            const float2 R0 = counts2(b0, p, K[PK_BIAS]), R1 = counts2(b1, p, K[PK_BIAS]);
            float2 y = fma2(X2, fma2(R1, K[PK_K2325], mul2(R0, K[PK_K12])), mul2(R1, K[PK_K21]));
            // RyR states 3/4: lumped above 3.685e-2
            const bool h0 = X.x > 3.685e-2f, h1 = X.y > 3.685e-2f;
            const float2 R2 = counts2(b2, p, K[PK_BIAS]), R3 = counts2(b3, p, K[PK_BIAS]);
            float2 p34 = fma2(R2, K[PK_K32], fma2(R3, K[PK_K4543], mul2(mul2(X2, R2), K[PK_K34])));
            if (h0 || h1) {
                const float2 num = fma2(K[PK_K45K34], X2, K[PK_K32K43]), den = fma2(K[PK_K34], X2, K[PK_K43]);
                const float2 hv = mul2(add2(R2, R3), div2(num, den));
                if (h0) p34.x = hv.x;
                if (h1) p34.y = hv.y;
            }
            y = add2(y, p34);
            // RyR states 5/6: lumped above 1.15e-4
            const bool g0 = X.x > 1.15e-4f, g1 = X.y > 1.15e-4f;
            const float2 R4 = counts2(b4, p, K[PK_BIAS]), R5 = counts2(b5, p, K[PK_BIAS]);
            float2 p56 = make_float2(0.f, 0.f);
            if (!(g0 && g1)) p56 = fma2(R5, K[PK_K65], fma2(R4, K[PK_K52], mul2(mul2(X2, R4), K[PK_K5654])));
            if (g0 || g1) {
                const float2 num = mul2(K[PK_K65], fma2(K[PK_K54], X2, K[PK_K52])), den = fma2(K[PK_K56], X2, K[PK_K65]);
                const float2 hv = mul2(add2(R4, R5), div2(num, den));
                if (g0) p56.x = hv.x;
                if (g1) p56.y = hv.y;
            }
            y = add2(y, p56);
            // LCC, gate and ClCh rates from the warp's table: base + slope * CaSS
            const float2 ta = tab[(iw >> (16 * p)) & 0x3Fu], tb = tab[(iw >> (16 * p + 8)) & 0x3Fu];
            Y[p] = y;
            S[p] = add2(make_float2(fmaf(ta.y, X.x, ta.x), fmaf(tb.y, X.y, tb.x)), y);
        }
        const float sub[4] = {S[0].x, S[0].y, S[1].x, S[1].y};
        const float2 st = add2(S[0], S[1]);
        const float total = st.x + st.y;
        const float u0 = rng.uniform<float>(k);
        const float jump = -logf(u0) * rcp_approx(total);
        const bool last = !(t + jump < dt);
        const float h = last ? (dt - t) : jump;

        // update_CaSS (SSA.tpp:87-99), first pass
        float2 tmp[2];
        const float2 H = make_float2(h, h);
#pragma unroll
        for (int p = 0; p < 2; ++p) {
            const float2 A = add2(K[PK_KBSR], C[p]), B = add2(K[PK_KBSL], C[p]);
            const float2 U = mul2(A, A), V = mul2(B, B);
            const float2 UV = mul2(U, V);
            const float2 den = fma2(K[PK_BSL], U, fma2(K[PK_BSR], V, UV));
            const float2 beta = div2(UV, den);
            const float2 jl = make_float2(s.jlcc[2 * p], s.jlcc[2 * p + 1]);
            const float2 jr = make_float2(jrel[2 * p], jrel[2 * p + 1]);
            const float2 f = add2(add2(add2(jl, jr), neg2(jx[p])), jiss[p]);
            tmp[p] = add2(C[p], mul2(mul2(H, f), beta));
        }
        // Threshold crossings are rare: an exact any-crossing test first, then the kinds and the
        // re-split draw count only when one occurred (if-converted, the full test per subunit
        // cost ~120 instructions per CRU-step).
        bool crossed = false;
#pragma unroll
        for (int p = 0; p < 2; ++p) {
            crossed |= (C[p].x > 1.15e-4f && tmp[p].x <= 1.15e-4f) || (C[p].x > 0.03685f && tmp[p].x <= 0.03685f);
            crossed |= (C[p].y > 1.15e-4f && tmp[p].y <= 1.15e-4f) || (C[p].y > 0.03685f && tmp[p].y <= 0.03685f);
        }
        int kind[4] = {0, 0, 0, 0};
        uint32_t D = 0;
        if (crossed) {
            kind[0] = crossing<float>(s, 0, C[0].x, tmp[0].x, D);
            kind[1] = crossing<float>(s, 1, C[0].y, tmp[0].y, D);
            kind[2] = crossing<float>(s, 2, C[1].x, tmp[1].x, D);
            kind[3] = crossing<float>(s, 3, C[1].y, tmp[1].y, D);
        }

        uint32_t kk = k + 1u + D;
        int act = 0, aj = 0, atr = 0;
        if (!last) {
            t += jump;
            const float ryr_sub[4] = {Y[0].x, Y[0].y, Y[1].x, Y[1].y};
            select_event_f32(s, c, sv, sub, ryr_sub, total, rng, kk, act, aj, atr);
        }
        if (crossed) resplit_crossed<float>(s, c, kind, rng, k);
        s.cass[0] = tmp[0].x;
        s.cass[1] = tmp[0].y;
        s.cass[2] = tmp[1].x;
        s.cass[3] = tmp[1].y;

        // update_CaJSR (SSA.hpp:68-71), Fast2Sum into (hi, lo) as in the generic lane
        {
            const float x = s.cajsr;
            const float u = (c.KCSQN + x) * (c.KCSQN + x);
            const float beta = u * rcp_approx(u + c.CSQN_const);
            const float2 jr = add2(make_float2(jrel[0], jrel[1]), make_float2(jrel[2], jrel[3]));
            const float d = h * beta * (jtr - c.VSS_VJSR * (jr.x + jr.y));
            const float hi = s.cajsr;
            const float y = d + s.cajsr_lo;
            const float sum = hi + y;
            const float err_ = y - (sum - hi);
            s.cajsr = sum;
            s.cajsr_lo = err_;
        }

        if (act != 0) apply_event<float>(s, c, sv, act, aj, atr, jrel);
        const float2 jxs = add2(jx[0], jx[1]);
        jxfer_sum = jxs.x + jxs.y;
        k = kk;
        if (last) return true;
        if (++ev > cap) {
            err = 1;
            return true;
        }
        return false;
    }
};

template <typename R, bool EXACT>
__device__ __forceinline__ void ssa_cru(Cru<R> &s, const SsaConsts<R> &c, const R *sv, const float2 *tab, Stream &rng,
                                        R dt, int cap, R &out_jxfer, R &out_jtr, int &events,
                                        int &err) {
    SsaLane<R, EXACT> L;
    L.begin(s, c);
    while (!L.iterate(s, c, sv, tab, rng, dt, cap, err)) {
    }
    events += L.ev;
    out_jxfer = L.jxfer_sum;
    out_jtr = L.jtr;
}

}  // namespace dev
}  // namespace gw
