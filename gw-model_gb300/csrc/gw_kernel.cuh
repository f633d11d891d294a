// gw_kernel.cuh -- the GB300 engine kernel for the Greenstein-Winslow hybrid SSA.
//
// One launch advances every cell of an ensemble by n_steps global steps.  A cell's CRUs are
// spread over the CTAs of one thread-block cluster; each CTA keeps its CRU tile in shared memory
// for the whole launch (no HBM traffic per step).  Per global step n:
//
//   SSA warps   : per-CRU hybrid SSA of step n (SSA.tpp:286-310) with V, Cai, CaNSR of step n,
//                 then per-warp flux partials pushed into the leader CTA's shared memory (DSMEM).
//   ODE warp    : (leader CTA of each cell only, concurrently with the SSA warps) reduces the
//                 partials of step n-1 and takes the FP64 global step n -> n+1
//                 (GW.tpp:237-272), then pushes the per-step SSA values of step n+1 to every CTA
//                 of the cell.
//   one barrier.cluster per step separates producers and consumers (double-buffered slots).
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
__device__ __forceinline__ void st_remote(uint32_t addr, double v) {
    asm volatile("st.shared::cluster.f64 [%0], %1;" ::"r"(addr), "d"(v) : "memory");
}
__device__ __forceinline__ void st_remote(uint32_t addr, float v) {
    asm volatile("st.shared::cluster.f32 [%0], %1;" ::"r"(addr), "f"(v) : "memory");
}

// ------------------------------------------------------------------------------------------
// Per-cell SSA constants (shared memory, in the CRU arithmetic type).
// ------------------------------------------------------------------------------------------
template <typename R>
struct SsaConsts {
    R k12, k21, k23, k32, k34, k43, k45, k54, k56, k65, k25, k52;
    R rRyR, rxfer, rtr, riss, KBSR, KBSL, KCSQN, kfClCh, kbClCh;
    R BSR_const, BSL_const, VSS_VJSR, CSQN_const, Cao_scaled;
    R gam[5];  // gamma0 * a^k, k = 0..4 (Constants gamma0 .. gamma0a4)
    R pad;
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
    c.pad = (R)0;
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
    const uint32_t w = lcc_table(st);
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

struct CruOut {
    float jxfer, jtr;   // FP32 path
    double jxfer_d, jtr_d;
    int events;
    int err;
};

// One CRU over one global step: SSA_single_CRU (SSA.tpp:286-310) with the reference's draw order.
// The jump draw comes first; then update_CaSS's binomial re-splits (sample_RyR56/34), then the
// subunit and transition draws.  The transition is chosen from the rates of the start of the
// iteration (as the reference's stored rate arrays are) and applied after the Ca update, so the
// code reorders independent work but not values: re-split draws use indices k+1..k+D and the
// selection draws k+D+1.. exactly as the reference's sequential urand() calls would.
template <typename R, bool EXACT>
__device__ __forceinline__ void ssa_cru(Cru<R> &s, const SsaConsts<R> &c, const R *sv, Stream &rng,
                                        R dt, int cap, R &out_jxfer, R &out_jtr, int &events,
                                        int &err) {
    int ev = 0;
    const R Cai = sv[SV_CAI], CaNSR = sv[SV_CANSR];
    const R Cai_lo = EXACT ? (R)0 : sv[SV_CAI_LO], CaNSR_lo = EXACT ? (R)0 : sv[SV_CANSR_LO];
    R jrel[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const R open = (R)(byte_s(s.ryr[2], j) + byte_s(s.ryr[3], j));
        jrel[j] = c.rRyR * open * (s.cajsr - s.cass[j]);
    }
    R t = (R)0;
    uint32_t k = 0;
    R jxfer[4], jiss[4], jtr;
    for (;;) {
        // update_fluxes (SSA.tpp:37-45)
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
        // update_rates (SSA.tpp:48-56): only the subunit totals are kept here.
        R sub[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            Rates<R> r;
            sub[j] = subunit_rates<R>(s, j, s.cass[j], c, sv, r);
        }
        const R total = sub[0] + sub[1] + sub[2] + sub[3];
        const R u0 = rng.uniform<R>(k);
        R jump;
        if (EXACT)
            jump = -log(u0) / total;
        else
            jump = -logf((float)u0) / (float)total;
        const bool last = !(t + jump < dt);
        const R h = last ? (dt - t) : jump;

        // update_CaSS (SSA.tpp:87-99), first pass: new values and threshold crossings.
        R tmp[4];
        int kind[4];
        uint32_t D = 0;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const R x = s.cass[j];
            R beta;
            if (EXACT) {
                beta = (R)1.0 / ((R)1 + (c.BSR_const / ((c.KBSR + x) * (c.KBSR + x))) +
                                 (c.BSL_const / ((c.KBSL + x) * (c.KBSL + x))));
            } else {
                const R u = (c.KBSR + x) * (c.KBSR + x), v = (c.KBSL + x) * (c.KBSL + x);
                const R uv = u * v;
                beta = __fdividef((float)uv, (float)(uv + c.BSR_const * v + c.BSL_const * u));
            }
            const R d = h * (s.jlcc[j] + jrel[j] - jxfer[j] + jiss[j]) * beta;
            tmp[j] = x + d;
            kind[j] = 0;
            if (x > (R)1.15e-4 && tmp[j] <= (R)1.15e-4) {
                kind[j] = 1;
                const int n = byte_s(s.ryr[4], j) + byte_s(s.ryr[5], j);
                if (n > 0) D += (uint32_t)n;
            } else if (x > (R)0.03685 && tmp[j] <= (R)0.03685) {
                kind[j] = 2;
                const int n = byte_s(s.ryr[2], j) + byte_s(s.ryr[3], j);
                if (n > 0) D += (uint32_t)n;
            }
        }

        // Event selection (sample_weights over subunits, sample_new_state) from the rates of the
        // start of this iteration, with draws k+D+1, k+D+2, k+D+3.
        uint32_t kk = k + 1u + D;
        int act = 0;      // 0 none, 1 LCC, 2 inactivation toggle, 3 RyR, 4 ClCh toggle
        int aj = 0, atr = 0;
        if (!last) {
            t += jump;
            const R us = rng.uniform<R>(kk++) * total;
            aj = scan_weights<R, 4, !EXACT>(sub, us);
            Rates<R> r;
            const R sr = subunit_rates<R>(s, aj, pick4(s.cass, aj), c, sv, r);
            (void)sr;
            const R subr = pick4(sub, aj);
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

        // update_CaSS second pass: binomial re-splits (sample_RyR56/34, SSA.tpp:59-84) with draws
        // k+1 .. k+D, then commit.
        if (D > 0 || kind[0] || kind[1] || kind[2] || kind[3]) {
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
#pragma unroll
        for (int j = 0; j < 4; ++j) s.cass[j] = tmp[j];

        // update_CaJSR (SSA.hpp:68-71)
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

        // Apply the transition (sample_new_state, SSA.tpp:262-283) to the updated state.
        if (act != 0) {
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                if (j != aj) continue;
                if (act == 1) {
                    const int from = byte_u(s.lcc, j);
                    if (from >= 1 && from <= 12) {
                        const int to = lcc_next(from, atr);
                        s.lcc = byte_set(s.lcc, j, to);
                        const bool inact1 = ((s.flags >> j) & 1u) != 0u;
                        if ((from == 5 && to == 6) || (from == 11 && to == 12))
                            s.jlcc[j] = inact1 ? sv[SV_JMUL] * (c.Cao_scaled - sv[SV_JEXP] * s.cass[j]) : (R)0;
                        else if (from == 6 || from == 12)
                            s.jlcc[j] = (R)0;
                    }
                } else if (act == 2) {
                    s.flags ^= (1u << j);
                    const int st = byte_u(s.lcc, j);
                    if (((s.flags >> j) & 1u) == 0u)
                        s.jlcc[j] = (R)0;
                    else if (st == 6 || st == 12)
                        s.jlcc[j] = sv[SV_JMUL] * (c.Cao_scaled - sv[SV_JEXP] * s.cass[j]);
                } else if (act == 3) {
                    int from, to;
                    ryr_move(atr, from, to);
#pragma unroll
                    for (int q = 0; q < 6; ++q) {
                        if (q == from) s.ryr[q] = byte_add(s.ryr[q], j, -1);
                        if (q == to) s.ryr[q] = byte_add(s.ryr[q], j, +1);
                    }
                    const R open = (R)(byte_s(s.ryr[2], j) + byte_s(s.ryr[3], j));
                    jrel[j] = c.rRyR * open * (s.cajsr - s.cass[j]);
                } else {
                    s.flags ^= (1u << (4 + j));
                }
            }
        }
        k = kk;
        if (last) break;
        if (++ev > cap) {
            err = 1;
            break;
        }
    }
    events += ev;
    out_jxfer = jxfer[0] + jxfer[1] + jxfer[2] + jxfer[3];
    out_jtr = jtr;
}

// ------------------------------------------------------------------------------------------
// Global step (GW_model::euler_step, GW.tpp:237-272) for one cell, evaluated by one thread.
// T is the arithmetic of the right-hand side: double (reference semantics) or float (optional
// mixed mode); the state and its Euler update are always FP64.  With T = double the expressions
// follow the reference's order term by term.
// ------------------------------------------------------------------------------------------
enum { GI_V = 0, GI_Nai, GI_Ki, GI_Cai, GI_CaNSR, GI_CaLTRPN, GI_CaHTRPN, GI_m, GI_h, GI_j, GI_xKs,
       GI_Kr = 11, GI_Kv43 = 16, GI_Kv14 = 26 };

__device__ __forceinline__ double t_exp(double x) { return exp(x); }
__device__ __forceinline__ float t_exp(float x) { return expf(x); }
__device__ __forceinline__ double t_log(double x) { return log(x); }
__device__ __forceinline__ float t_log(float x) { return logf(x); }
__device__ __forceinline__ double t_pow(double x, double y) { return pow(x, y); }
__device__ __forceinline__ float t_pow(float x, float y) { return powf(x, y); }

// Generator entries of one 10-state Kv channel (update_QKv, GW.tpp:65-123) and its derivative
// (update_Kv_derivatives, GW.tpp:136-160).
template <typename T>
__device__ __forceinline__ void kv_derivs(const double *xs_, T aa, T ai, T ba, T bi, T f1, T f2,
                                          T f3, T f4, T b1, T b2, T b3, T b4, T dt, T *d) {
    const T q01 = 4 * aa, q05 = bi, q00 = -(q01 + q05);
    const T q10 = ba, q12 = 3 * aa, q16 = f1 * bi, q11 = -(q10 + q12 + q16);
    const T q21 = 2 * ba, q23 = 2 * aa, q27 = f2 * bi, q22 = -(q21 + q23 + q27);
    const T q32 = 3 * ba, q34 = aa, q38 = f3 * bi, q33 = -(q32 + q34 + q38);
    const T q43 = 4 * ba, q49 = f4 * bi, q44 = -(q43 + q49);
    const T q56 = 4 * aa * b1, q50 = ai, q55 = -(q56 + q50);
    const T q65 = ba / f1, q67 = 3 * aa * b2 / b1, q61 = ai / b1, q66 = -(q65 + q67 + q61);
    const T q76 = 2 * ba * f1 / f2, q78 = 2 * aa * b3 / b2, q72 = ai / b2, q77 = -(q76 + q78 + q72);
    const T q87 = 3 * ba * f2 / f3, q89 = aa * b4 / b3, q83 = ai / b3, q88 = -(q87 + q89 + q83);
    const T q98 = 4 * ba * f3 / f4, q94 = ai / b4, q99 = -(q98 + q94);
    const T x0 = (T)xs_[0], x1 = (T)xs_[1], x2 = (T)xs_[2], x3 = (T)xs_[3], x4 = (T)xs_[4];
    const T x5 = (T)xs_[5], x6 = (T)xs_[6], x7 = (T)xs_[7], x8 = (T)xs_[8], x9 = (T)xs_[9];
    d[0] = dt * (q10 * x1 + q50 * x5 + q00 * x0);
    d[1] = dt * (q01 * x0 + q21 * x2 + q61 * x6 + q11 * x1);
    d[2] = dt * (q12 * x1 + q32 * x3 + q72 * x7 + q22 * x2);
    d[3] = dt * (q23 * x2 + q43 * x4 + q83 * x8 + q33 * x3);
    d[4] = dt * (q34 * x3 + q94 * x9 + q44 * x4);
    d[5] = dt * (q65 * x6 + q05 * x0 + q55 * x5);
    d[6] = dt * (q56 * x5 + q76 * x7 + q16 * x1 + q66 * x6);
    d[7] = dt * (q67 * x6 + q87 * x8 + q27 * x2 + q77 * x7);
    d[8] = dt * (q78 * x7 + q98 * x9 + q38 * x3 + q88 * x8);
    d[9] = dt * (q89 * x8 + q49 * x4 + q99 * x9);
}

// One global step of one cell.  g: the 36 globals (updated in place).  sums: JLCC, ClCh, Jtr,
// Jxfer sums of the previous step's SSA.  expm = exp(-V F/RT) of the current V.  Returns 0 or a
// gw_status code (GW_ERR_NERNST where the reference would exit).
template <typename T>
__device__ __noinline__ int ode_step(const CellStatic &C, double *g, const double *sums, double Istim_,
                        double dt_, double expm_) {
    const gw_params &p = C.p;
    const T V = (T)g[GI_V], Nai = (T)g[GI_Nai], Ki = (T)g[GI_Ki], Cai = (T)g[GI_Cai];
    const T CaNSR = (T)g[GI_CaNSR], CaLTRPN = (T)g[GI_CaLTRPN], CaHTRPN = (T)g[GI_CaHTRPN];
    const T m = (T)g[GI_m], h = (T)g[GI_h], j = (T)g[GI_j], xKs = (T)g[GI_xKs];
    const T dt = (T)dt_, Istim = (T)Istim_;
    const T RT_F = (T)C.RT_F, F_RT = (T)C.F_RT;
    const T VF_RT = V * F_RT;
    const T expm = (T)expm_;
    int status = 0;
    if (!(Nai > (T)0) || !(Ki > (T)0)) status = GW_ERR_NERNST;
    // update_V_and_concentration_derivatives (GW.tpp:171-212)
    const T ENa = t_log((T)p.Nao / Nai) * RT_F / (T)1.0;
    const T EK = t_log((T)p.Ko / Ki) * RT_F / (T)1.0;
    const T ECa = t_log((T)p.Ko / Ki) * RT_F / (T)2.0;
    const T INa = (T)p.GNa * (m * m * m) * h * j * (V - ENa);
    const T INab = (T)p.GNab * (V - ENa);
    T INaCa;
    {
        const T e1 = t_exp((T)p.eta * VF_RT);
        const T e2 = e1 * expm;
        INaCa = (T)C.INaCa_const * (e1 * (Nai * Nai * Nai) * (T)p.Cao - e2 * (T)C.Nao3 * Cai) /
                ((T)1.0 + (T)p.ksat * e2);
    }
    T INaK;
    {
        const T fNaK = (T)1.0 / ((T)1.0 + (T)0.1245 * t_exp((T)-0.1 * VF_RT) +
                                 (T)0.0365 * (T)C.sigma * expm);
        INaK = (T)C.INaK_const * fNaK / ((T)1.0 + t_pow((T)p.KmNai / Nai, (T)1.5));
    }
    T IKr;
    {
        const T RKr = (T)1.0 / ((T)1.0 + (T)1.4945 * t_exp((T)0.0446 * V));
        IKr = (T)p.GKr * (T)C.sqrtKo * RKr * (T)g[GI_Kr + 3] * (V - EK) * (T)0.5;
    }
    T IKs;
    {
        const T EKs = t_log(((T)p.Ko + (T)0.01833 * (T)p.Nao) / (Ki + (T)0.01833 * Nai)) * RT_F;
        IKs = (T)p.GKs * (xKs * xKs) * (V - EKs);
    }
    T Ito1;
    {
        const T mm = ((T)C.PKv14_Csc) * ((T)kFaraday * VF_RT) * (T)g[GI_Kv14 + 4] / ((T)1 - expm);
        const T IKv14 = mm * ((Ki - (T)p.Ko * expm) + (T)0.02 * (Nai - (T)p.Nao * expm)) * (T)1.0e9;
        const T IKv43 = (T)p.GKv43 * (T)g[GI_Kv43 + 4] * (V - EK);
        Ito1 = IKv14 + IKv43;
    }
    const T Ito2 = (T)sums[1] * (T)C.Ito2_const * VF_RT * ((T)p.Clcyto * expm - (T)p.Clo) /
                   (expm - (T)1.0);
    T IK1;
    {
        const T K1inf = (T)1.0 / ((T)2.0 + t_exp((T)1.5 * (V - EK) * F_RT));
        IK1 = (T)p.GK1 * K1inf * (T)C.IK1_const * (V - EK);
    }
    T IKp;
    {
        const T Kp = (T)1. / ((T)1. + t_exp(((T)7.488 - V) / (T)5.98));
        IKp = (T)p.GKp * Kp * (V - EK);
    }
    const T ICaL = (T)sums[0] * (T)C.ICaL_const;
    const T ICab = (T)p.GCab * (V - ECa);
    const T IpCa = (T)p.IpCamax * (Cai / ((T)p.KmpCa + Cai));
    T Jup;
    {
        const T f = t_pow(Cai / (T)p.Kmf, (T)p.Hf);
        const T r = t_pow(CaNSR / (T)p.Kmr, (T)p.Hr);
        Jup = ((T)p.Vmaxf * f - (T)p.Vmaxr * r) / ((T)1.0 + f + r);
    }
    const T Jtr_tot = (T)sums[2] * (T)C.CRU_factor;
    const T Jxfer_tot = (T)sums[3] * (T)C.CRU_factor;
    T beta_cyto;
    {
        const T x = (T)p.KCMDN + Cai;
        beta_cyto = (T)1.0 / ((T)1.0 + (T)C.CMDN_const / (x * x));
    }
    T dLTRPN = (T)p.kLTRPNp * Cai * ((T)p.LTRPNtot - CaLTRPN) - (T)p.kLTRPNm * CaLTRPN;
    T dHTRPN = (T)p.kHTRPNp * Cai * ((T)p.HTRPNtot - CaHTRPN) - (T)p.kHTRPNm * CaHTRPN;
    const T CSA_FVcyto = (T)C.CSA_FVcyto;
    const T dNai = -dt * CSA_FVcyto * (INa + INab + (T)3 * INaCa + (T)3 * INaK);
    const T dKi = -dt * CSA_FVcyto * (IKr + IKs + Ito1 + IK1 + IKp - (T)2 * INaK);
    const T dCai = dt * beta_cyto *
                   ((T)-0.5 * CSA_FVcyto * (ICab + IpCa - (T)2 * INaCa) +
                    (T)C.VSS_Vcyto * Jxfer_tot - Jup - (dLTRPN + dHTRPN));
    const T dCaNSR = dt * ((T)C.Vcyto_VNSR * Jup - (T)C.VJSR_VNSR * Jtr_tot);
    dLTRPN *= dt;
    dHTRPN *= dt;
    const T dV = dt * (Istim - (INa + ICaL + IKr + IKs + Ito1 + IK1 + IKp + Ito2 + INaK + INaCa +
                                IpCa + ICab + INab));
    // update_gate_derivatives (GW.tpp:163-168)
    T dm, dh, dj, dxKs;
    {
        const T am = (V == (T)-47.13) ? (T)3.2
                                      : (T)0.32 * (V + (T)47.13) /
                                            ((T)1.0 - t_exp((T)-0.1 * (V + (T)47.13)));
        const T bm = (T)0.08 * t_exp(-V / (T)11.0);
        const T ah = (V >= (T)-40.0) ? (T)0.0 : (T)0.135 * t_exp(-(V + (T)80.0) / (T)6.8);
        const T bh = (V >= (T)-40.0)
                         ? (T)1.0 / ((T)0.13 * ((T)1.0 + t_exp(-(V + (T)10.66) / (T)11.1)))
                         : (T)3.56 * t_exp((T)0.079 * V) + (T)3.1e5 * t_exp((T)0.35 * V);
        const T aj = (V >= (T)-40.0)
                         ? (T)0.0
                         : ((T)-127140.0 * t_exp((T)0.2444 * V) -
                            (T)3.474e-5 * t_exp((T)-0.04391 * V)) *
                               (V + (T)37.78) / ((T)1.0 + t_exp((T)0.311 * (V + (T)79.23)));
        const T bj = (V >= (T)-40.0)
                         ? (T)0.3 * t_exp((T)-2.535e-7 * V) /
                               ((T)1.0 + t_exp((T)-0.1 * (V + (T)32.0)))
                         : (T)0.1212 * t_exp((T)-0.01052 * V) /
                               ((T)1.0 + t_exp((T)-0.1378 * (V + (T)40.14)));
        const T xinf = (T)1.0 / ((T)1.0 + t_exp(-(V - (T)24.7) / (T)13.6));
        const T tinv = (T)0.0000719 * (V - (T)10.0) / ((T)1.0 - t_exp((T)-0.148 * (V - (T)10.0))) +
                       (T)0.000131 * (V - (T)10.0) / (t_exp((T)0.0687 * (V - (T)10.0)) - (T)1.0);
        dm = dt * (am * ((T)1.0 - m) - bm * m);
        dh = dt * (ah * ((T)1.0 - h) - bh * h);
        dj = dt * (aj * ((T)1.0 - j) - bj * j);
        dxKs = dt * (xinf - xKs) * tinv;
    }
    // update_QKr + update_Kr_derivatives (GW.tpp:26-44, 127-133)
    T dKr[5];
    {
        const T Q01 = (T)0.0069 * t_exp((T)0.0272 * V);
        const T Q00 = -Q01;
        const T Q10 = (T)0.0227 * t_exp((T)-0.0431 * V);
        const T Q12 = (T)p.Kf, Q21 = (T)p.Kb;
        const T Q11 = -(Q10 + Q12);
        const T Q23 = (T)0.0218 * t_exp((T)0.0262 * V);
        const T Q24 = (T)1.29e-5 * t_exp((T)2.71e-6 * V);
        const T Q22 = -(Q21 + Q23 + Q24);
        const T Q32 = (T)0.0009 * t_exp((T)-0.0269 * V);
        const T Q34 = (T)0.0622 * t_exp((T)0.0120 * V);
        const T Q33 = -(Q32 + Q34);
        const T Q43 = (T)0.0059 * t_exp((T)-0.0443 * V);
        const T Q42 = Q32 * Q43 * Q24 / (Q23 * Q34);
        const T Q44 = -(Q42 + Q43);
        T k[5];
#pragma unroll
        for (int i = 0; i < 5; ++i) k[i] = (T)g[GI_Kr + i];
        dKr[0] = dt * (Q10 * k[1] + Q00 * k[0]);
        dKr[1] = dt * (Q01 * k[0] + Q21 * k[2] + Q11 * k[1]);
        dKr[2] = dt * (Q12 * k[1] + Q32 * k[3] + Q42 * k[4] + Q22 * k[2]);
        dKr[3] = dt * (Q23 * k[2] + Q43 * k[4] + Q33 * k[3]);
        dKr[4] = dt * (Q24 * k[2] + Q34 * k[3] + Q44 * k[4]);
    }
    T dKv14[10], dKv43[10];
    {
        const T aa14 = (T)p.alphaa0Kv14 * t_exp((T)p.aaKv14 * V);
        const T aa43 = (T)p.alphaa0Kv43 * t_exp((T)p.aaKv43 * V);
        const T ai14 = (T)p.alphai0Kv14 * t_exp(-(T)p.aiKv14 * V);
        const T ai43 = (T)p.alphai0Kv43 * t_exp(-(T)p.aiKv43 * V);
        const T ba14 = (T)p.betaa0Kv14 * t_exp(-(T)p.baKv14 * V);
        const T ba43 = (T)p.betaa0Kv43 * t_exp(-(T)p.baKv43 * V);
        const T bi14 = (T)p.betai0Kv14 * t_exp((T)p.biKv14 * V);
        const T bi43 = (T)p.betai0Kv43 * t_exp((T)p.biKv43 * V);
        kv_derivs<T>(g + GI_Kv14, aa14, ai14, ba14, bi14, (T)p.f1Kv14, (T)p.f2Kv14, (T)p.f3Kv14,
                     (T)p.f4Kv14, (T)p.b1Kv14, (T)p.b2Kv14, (T)p.b3Kv14, (T)p.b4Kv14, dt, dKv14);
        kv_derivs<T>(g + GI_Kv43, aa43, ai43, ba43, bi43, (T)p.f1Kv43, (T)p.f2Kv43, (T)p.f3Kv43,
                     (T)p.f4Kv43, (T)p.b1Kv43, (T)p.b2Kv43, (T)p.b3Kv43, (T)p.b4Kv43, dt, dKv43);
    }
    // Euler update (GW.tpp:252-271), accumulated in FP64.
    g[GI_V] += (double)dV;
    g[GI_Nai] += (double)dNai;
    g[GI_Ki] += (double)dKi;
    g[GI_Cai] += (double)dCai;
    g[GI_CaNSR] += (double)dCaNSR;
    g[GI_CaLTRPN] += (double)dLTRPN;
    g[GI_CaHTRPN] += (double)dHTRPN;
    g[GI_m] += (double)dm;
    g[GI_h] += (double)dh;
    g[GI_j] += (double)dj;
    g[GI_xKs] += (double)dxKs;
#pragma unroll
    for (int i = 0; i < 5; ++i) g[GI_Kr + i] += (double)dKr[i];
#pragma unroll
    for (int i = 0; i < 10; ++i) {
        g[GI_Kv14 + i] += (double)dKv14[i];
        g[GI_Kv43 + i] += (double)dKv43[i];
    }
    return status;
}

// Per-step SSA values at voltage V (GW_model::SSA, GW.tpp:216-221; alphaLCC..tauLCC,
// GW_utils.hpp:365-375) with the LCC rate products of update_LCC_rates.  Fills sv[0..33] and
// returns exp(-V F/RT), which the next global step uses as expmVF_RT.
static __device__ __noinline__ double step_values(const CellStatic &C, const double *g, double *sv) {
    const double V = g[GI_V];
    const double expm = exp(-(V * C.F_RT));
    const double al = 2.0 * exp(0.012 * (V - 35.0));
    const double be = 0.0882 * exp(-0.05 * (V - 35.0));
    const double yinf = 0.4 / (1.0 + exp((V + 12.5) / 5.0)) + 0.6;
    const double tau = 340.0 / (1.0 + exp((V + 30.0) / 12.0)) + 60.0;
    const gw_params &p = C.p;
    sv[SV_ZERO] = 0.0;
    sv[SV_A4] = 4 * al; sv[SV_A3] = 3 * al; sv[SV_A2] = 2 * al; sv[SV_A1] = al;
    sv[SV_B1] = be; sv[SV_B2] = 2 * be; sv[SV_B3] = 3 * be; sv[SV_B4] = 4 * be;
    sv[SV_A4a] = 4 * al * C.a; sv[SV_A3a] = 3 * al * C.a; sv[SV_A2a] = 2 * al * C.a;
    sv[SV_A1a] = al * C.a;
    sv[SV_B1bi] = be * C.binv; sv[SV_B2bi] = 2 * be * C.binv; sv[SV_B3bi] = 3 * be * C.binv;
    sv[SV_B4bi] = 4 * be * C.binv;
    sv[SV_F] = p.f; sv[SV_G] = p.g; sv[SV_OM] = C.omega; sv[SV_OMB1] = C.omega_b;
    sv[SV_OMB2] = C.omega_b2; sv[SV_OMB3] = C.omega_b3; sv[SV_OMB4] = C.omega_b4;
    sv[SV_F1] = p.f1; sv[SV_G1] = p.g1;
    sv[SV_INACT0] = yinf / tau;
    sv[SV_INACT1] = (1.0 - yinf) / tau;
    const double jexp = (1.0 / expm) * (1.0 / expm);
    sv[SV_JEXP] = jexp;
    sv[SV_JMUL] = C.JLCC_const * V * C.F_RT / (jexp - 1);
    sv[SV_CAI] = g[GI_Cai];
    sv[SV_CANSR] = g[GI_CaNSR];
    sv[SV_CAI_LO] = 0.0;
    sv[SV_CANSR_LO] = 0.0;
    return expm;
}

}  // namespace dev
}  // namespace gw
