// gw_ode_program.cpp -- builds the SIMT lane program of the global step (see gw_ode_program.h).
//
// Every term below restates GW_model::euler_step (GW.tpp:237-272) and the functions it calls
// (update_V_and_concentration_derivatives GW.tpp:171-212, update_QKr/QKv GW.tpp:26-44/65-123,
// update_*_derivatives GW.tpp:127-168, the currents of common.hpp:70-218 and GW_utils.hpp:273-375,
// and the per-step constants of GW_model::SSA GW.tpp:216-221), rearranged into
//   phase E  SUMU : increments of the 36 globals (linear combinations of current / rate terms)
//                   and the Euler update g += dg (FP64) by each row's first lane; the rows read
//                   the old globals (X[XS_G]), the new ones go to X[XS_GN]
//   phase A  LOG | EXP | SQRT : transcendental terms of the new globals
//   phase B  AFF | REC | PROD | SQRT : reversal-potential differences, reciprocals, LCC rate table
//   phase C  PROD | REC | SUM | EXP : current terms, inactivation rates, JLCC factors
//   phase C2 REC  : (only with general Jup exponents) 1/(1 + f + r)
// The per-step SSA values are pushed after phase C.  Three V regimes select the branches of the
// gate rates (common.hpp:176-218): 0: V >= -40, 1: V < -40, 2: V == -47.13.
#include "gw_ode_program.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <utility>
#include <string>
#include <vector>

namespace gw {
namespace {

constexpr double kF = 96.5;  // common.hpp:9

struct Builder {
    const CellStatic &C;
    const gw_params &p;
    bool fast;
    int regime;
    double *consts;
    int const_begin;
    int nconst = 0;
    int next = XS_FIRST_FREE + kOdeMaxConsts;  // intermediates after the constant block
    std::vector<std::vector<OdeOp>> ph;
    std::vector<int> cursor;
    uint16_t sv_src[kSvCount];

    Builder(const CellStatic &c, bool f, int r, double *k)
        : C(c), p(c.p), fast(f), regime(r), consts(k), const_begin(XS_FIRST_FREE) {
        for (auto &s : sv_src) s = XS_ZERO;
    }

    // per-cell constant (allocated in call order, identical for every cell and regime)
    uint16_t K(double v) {
        const int i = nconst++;
        if (consts && i < kOdeMaxConsts) consts[i] = v;
        return (uint16_t)(const_begin + i);
    }
    // literal constant (same value for every cell): shared slot
    std::vector<std::pair<double, uint16_t>> lits;
    uint16_t KL(double v) {
        for (auto &l : lits)
            if (l.first == v) return l.second;
        const uint16_t s = K(v);
        lits.push_back({v, s});
        return s;
    }
    uint16_t S() { return (uint16_t)next++; }
    // Global i as read by the phase being built: the updated value (XS_GN) in the phases after
    // the update, the old value (XS_G) in the increments.
    bool post = true;
    uint16_t G(int i) const { return (uint16_t)((post ? XS_GN : XS_G) + i); }
    // increments emit OK_SUMU rows (out = global index) instead of OK_SUM
    bool upd_rows = false;

    void phase(int n) {
        ph.assign(n, {});
        cursor.assign(n, 0);
    }
    // start a new kind group at the next warp boundary of phase q
    void warp_align(int q) {
        auto &v = ph[q];
        while (v.size() % 32 != 0) v.push_back(OdeOp{OK_NOP, 1, 0, {}});
    }
    void emit(int q, uint8_t kind, uint16_t out, std::initializer_list<uint16_t> args, int width = 1) {
        auto &v = ph[q];
        while (v.size() % width != 0) v.push_back(OdeOp{OK_NOP, 1, 0, {}});
        OdeOp op{};
        op.kind = kind;
        op.width = (uint8_t)width;
        op.out = out;
        int i = 0;
        for (uint16_t a : args) op.a[i++] = a;
        for (; i < 14; ++i) op.a[i] = (kind == OK_PROD || kind == OK_SQRT) ? XS_ONE : XS_ZERO;
        if (kind == OK_EXP && args.size() < 4) op.a[3] = XS_ZERO;
        v.push_back(op);
    }
    // SUM row: out = s0 * s1 * sum(w * x * y); terms are padded to 4 per lane
    struct Term {
        uint16_t w, x, y;
    };
    void sum_row(int q, uint16_t out, uint16_t s0, uint16_t s1, std::vector<Term> terms) {
        int width = 1;
        while (width * 4 < (int)terms.size()) width *= 2;
        auto &v = ph[q];
        while (v.size() % width != 0) v.push_back(OdeOp{OK_NOP, 1, 0, {}});
        for (int l = 0; l < width; ++l) {
            OdeOp op{};
            op.kind = upd_rows ? OK_SUMU : OK_SUM;
            op.width = (uint8_t)width;
            op.out = out;
            op.a[0] = s0;
            op.a[1] = s1;
            for (int t = 0; t < 4; ++t) {
                const int k = l * 4 + t;
                const Term tm = k < (int)terms.size() ? terms[k] : Term{XS_ZERO, XS_ZERO, XS_ZERO};
                op.a[2 + 3 * t] = tm.w;
                op.a[3 + 3 * t] = tm.x;
                op.a[4 + 3 * t] = tm.y;
            }
            v.push_back(op);
        }
    }
};

enum { PH_E = 0, PH_F, PH_A, PH_B, PH_C, PH_C2, PH_COUNT };

void build(Builder &b) {
    const CellStatic &C = b.C;
    const gw_params &p = b.p;
    const int r = b.regime;
    const bool r0 = r == 0;  // V >= -40
    b.phase(PH_COUNT);
    const uint16_t ONE = XS_ONE, ZERO = XS_ZERO, MONE = XS_MONE;
    enum { iV = 0, iNai, iKi, iCai, iCaNSR, iCaL, iCaH, im, ih, ij, ixKs, iKr = 11, iKv43 = 16, iKv14 = 26 };
    const uint16_t V = b.G(iV), Nai = b.G(iNai), Ki = b.G(iKi), Cai = b.G(iCai), NSR = b.G(iCaNSR);
    const uint16_t SJLCC = XS_SUMS + 0, SClCh = XS_SUMS + 1, SJtr = XS_SUMS + 2, SJxfer = XS_SUMS + 3;
    // intermediates
    auto S = [&]() { return b.S(); };
    const uint16_t L_Na = S(), L_K = S(), L_Ks = S(), L_Cai = S(), L_NSR = S();
    const uint16_t NaS = S(), KiS = S(), s1f = S(), s1r = S(), pf = S(), pr = S();
    const uint16_t E_expm = S(), E_e1 = S(), E_e12 = S(), E_e01 = S(), E_Kr = S(), E_Kp = S();
    const uint16_t Q01 = S(), Q10 = S(), Q23 = S(), Q24 = S(), Q32 = S(), Q34 = S(), Q43 = S();
    uint16_t kv[2][4];  // [Kv14, Kv43][aa, ai, ba, bi]
    for (auto &c : kv)
        for (auto &x : c) x = S();
    const uint16_t E_am = S(), E_bm = S(), E_ah = S(), E_bh1 = S(), E_bh2 = S(), E_aj1 = S(), E_aj2 = S(),
                   E_aj3 = S(), E_bj1 = S(), E_bj2 = S(), E_xinf = S(), E_t1 = S(), E_t2 = S(), E_K1V = S();
    const uint16_t E_al = S(), E_be = S(), E_y = S(), E_t = S();
    const uint16_t VmENa = S(), VmEK = S(), VmECa = S(), VmEKs = S(), Vp47 = S(), Vp37 = S(), Vm10 = S(),
                   LmL = S(), HmH = S(), KiNa02 = S(), argf = S(), argr = S();
    const uint16_t rKr = S(), rKp = S(), rfNaK = S(), rNaCa = S(), r1me = S(), ram = S(), rbh = S(), raj = S(),
                   rbj = S(), rxinf = S(), rt1 = S(), rt2 = S(), rIpCa = S(), rQ = S(), rC = S(), rK1 = S(),
                   rINaK = S(), ry = S(), rtau = S(), JEXP = S(), rj = S();
    const uint16_t A4 = S(), A3 = S(), A2 = S(), B2 = S(), B3 = S(), B4 = S(), A4a = S(), A3a = S(), A2a = S(),
                   A1a = S(), B1bi = S(), B2bi = S(), B3bi = S(), B4bi = S();
    const uint16_t T_INa = S(), T_INab = S(), T_NaCa1 = S(), T_NaCa2 = S(), P_NaK = S(), T_IKr = S(),
                   T_IKs = S(), T_Kv14a = S(), T_Kv14b = S(), T_Kv43 = S(), P_Ito2a = S(), P_Ito2b = S(),
                   T_IKp = S(), T_ICab = S(), T_IpCa = S(), T_dL1 = S(), T_dL2 = S(), T_dH1 = S(), T_dH2 = S(),
                   T_am = S(), T_aj1 = S(), T_aj2 = S(), T_bj = S(), T_t1 = S(), T_t2 = S(), Q42 = S(),
                   JMUL = S(), beta = S(), rJup = S(), INACT0 = S(), INACT1 = S();

    const double RT_F = C.RT_F, F_RT = C.F_RT;
    // ---------------- phase A: LOG | EXP | SQRT ----------------
    {
        const int q = PH_A;
        b.emit(q, OK_LOG, L_Na, {Nai, ZERO, ZERO});
        b.emit(q, OK_LOG, L_K, {Ki, ZERO, ZERO});
        b.emit(q, OK_LOG, L_Ks, {Ki, b.K(0.01833), Nai});
        if (!b.fast) {
            b.emit(q, OK_LOG, L_Cai, {Cai, ZERO, ZERO});
            b.emit(q, OK_LOG, L_NSR, {NSR, ZERO, ZERO});
        }
        b.warp_align(q);
        auto ex = [&](uint16_t out, uint16_t c, uint16_t a, uint16_t v, uint16_t bb) {
            b.emit(q, OK_EXP, out, {c, a, v, bb});
        };
        ex(E_expm, ONE, b.K(-F_RT), V, ZERO);
        ex(E_e1, ONE, b.K(p.eta * F_RT), V, ZERO);
        ex(E_e12, ONE, b.K((p.eta - 1.0) * F_RT), V, ZERO);
        ex(E_e01, ONE, b.K(-0.1 * F_RT), V, ZERO);
        ex(E_Kr, ONE, b.K(0.0446), V, ZERO);
        ex(E_Kp, ONE, b.K(-1.0 / 5.98), V, b.K(7.488 / 5.98));
        ex(Q01, b.K(0.0069), b.K(0.0272), V, ZERO);
        ex(Q10, b.K(0.0227), b.K(-0.0431), V, ZERO);
        ex(Q23, b.K(0.0218), b.K(0.0262), V, ZERO);
        ex(Q24, b.K(1.29e-5), b.K(2.71e-6), V, ZERO);
        ex(Q32, b.K(0.0009), b.K(-0.0269), V, ZERO);
        ex(Q34, b.K(0.0622), b.K(0.0120), V, ZERO);
        ex(Q43, b.K(0.0059), b.K(-0.0443), V, ZERO);
        ex(kv[0][0], b.K(p.alphaa0Kv14), b.K(p.aaKv14), V, ZERO);
        ex(kv[1][0], b.K(p.alphaa0Kv43), b.K(p.aaKv43), V, ZERO);
        ex(kv[0][1], b.K(p.alphai0Kv14), b.K(-p.aiKv14), V, ZERO);
        ex(kv[1][1], b.K(p.alphai0Kv43), b.K(-p.aiKv43), V, ZERO);
        ex(kv[0][2], b.K(p.betaa0Kv14), b.K(-p.baKv14), V, ZERO);
        ex(kv[1][2], b.K(p.betaa0Kv43), b.K(-p.baKv43), V, ZERO);
        ex(kv[0][3], b.K(p.betai0Kv14), b.K(p.biKv14), V, ZERO);
        ex(kv[1][3], b.K(p.betai0Kv43), b.K(p.biKv43), V, ZERO);
        // gate rates (common.hpp:176-218; GW_utils.hpp:358-362); constants allocated for every
        // regime so that the slot layout does not depend on it
        const uint16_t c0135 = b.K(0.135), c_ah = b.K(-1.0 / 6.8), c_ahb = b.K(-80.0 / 6.8);
        const uint16_t c_bh0a = b.K(-1.0 / 11.1), c_bh0b = b.K(-10.66 / 11.1);
        const uint16_t c356 = b.K(3.56), c0079 = b.K(0.079), c31e5 = b.K(3.1e5), c035 = b.K(0.35);
        const uint16_t c127 = b.K(-127140.0), c2444 = b.K(0.2444), c3474 = b.K(-3.474e-5), c04391 = b.K(-0.04391);
        const uint16_t c0311 = b.K(0.311), c0311b = b.K(0.311 * 79.23);
        const uint16_t c03 = b.K(0.3), c2535 = b.K(-2.535e-7), c01212 = b.K(0.1212), c01052 = b.K(-0.01052);
        const uint16_t cm01 = b.K(-0.1), cm32 = b.K(-3.2), c1378 = b.K(-0.1378), c1378b = b.K(-0.1378 * 40.14);
        ex(E_am, ONE, cm01, V, b.K(-4.713));
        ex(E_bm, b.K(0.08), b.K(-1.0 / 11.0), V, ZERO);
        if (r0) {
            ex(E_ah, ZERO, ZERO, V, ZERO);
            ex(E_bh1, ONE, c_bh0a, V, c_bh0b);
            ex(E_bh2, ZERO, ZERO, V, ZERO);
            ex(E_aj1, ZERO, ZERO, V, ZERO);
            ex(E_aj2, ZERO, ZERO, V, ZERO);
            ex(E_aj3, ONE, ZERO, V, ZERO);
            ex(E_bj1, c03, c2535, V, ZERO);
            ex(E_bj2, ONE, cm01, V, cm32);
        } else {
            ex(E_ah, c0135, c_ah, V, c_ahb);
            ex(E_bh1, c356, c0079, V, ZERO);
            ex(E_bh2, c31e5, c035, V, ZERO);
            ex(E_aj1, c127, c2444, V, ZERO);
            ex(E_aj2, c3474, c04391, V, ZERO);
            ex(E_aj3, ONE, c0311, V, c0311b);
            ex(E_bj1, c01212, c01052, V, ZERO);
            ex(E_bj2, ONE, c1378, V, c1378b);
        }
        ex(E_xinf, ONE, b.K(-1.0 / 13.6), V, b.K(24.7 / 13.6));
        ex(E_t1, ONE, b.K(-0.148), V, b.K(1.48));
        ex(E_t2, ONE, b.K(0.0687), V, b.K(-0.687));
        ex(E_K1V, ONE, b.K(1.5 * F_RT), V, ZERO);
        ex(E_al, b.K(2.0), b.K(0.012), V, b.K(-0.42));
        ex(E_be, b.K(0.0882), b.K(-0.05), V, b.K(1.75));
        ex(E_y, ONE, b.K(0.2), V, b.K(2.5));
        ex(E_t, ONE, b.K(1.0 / 12.0), V, b.K(2.5));
        while (b.ph[q].size() < 96) b.ph[q].push_back(OdeOp{OK_NOP, 1, 0, {}});
        // (KmNai/Nai)^1.5 = KmNai^1.5 / (Nai sqrt(Nai)); exp(1.5 F/RT (V - EK)) = exp(1.5 F/RT V) *
        // (Ki/Ko)^1.5 (EK = RT/F log(Ko/Ki)); (Cai/Kmf)^0.75 = s sqrt(s), s = sqrt(Cai/Kmf)
        b.emit(q, OK_SQRT, NaS, {ONE, Nai, Nai, ONE});
        b.emit(q, OK_SQRT, KiS, {b.K(std::pow(p.Ko, -1.5)), Ki, Ki, ONE});
        if (b.fast) {
            b.emit(q, OK_SQRT, s1f, {ONE, ONE, Cai, b.K(1.0 / p.Kmf)});
            b.emit(q, OK_SQRT, s1r, {ONE, ONE, NSR, b.K(1.0 / p.Kmr)});
        }
    }
    // ---------------- phase B: AFF | REC | PROD | SQRT ----------------
    {
        const int q = PH_B;
        auto aff = [&](uint16_t out, std::initializer_list<uint16_t> a) { b.emit(q, OK_AFF, out, a); };
        aff(VmENa, {V, ONE, L_Na, b.K(RT_F), ZERO, ZERO, b.K(-RT_F * std::log(p.Nao))});
        aff(VmEK, {V, ONE, L_K, b.K(RT_F), ZERO, ZERO, b.K(-RT_F * std::log(p.Ko))});
        aff(VmECa, {V, ONE, L_K, b.K(0.5 * RT_F), ZERO, ZERO, b.K(-0.5 * RT_F * std::log(p.Ko))});
        aff(VmEKs, {V, ONE, L_Ks, b.K(RT_F), ZERO, ZERO, b.K(-RT_F * std::log(p.Ko + 0.01833 * p.Nao))});
        aff(Vp47, {V, ONE, ZERO, ZERO, ZERO, ZERO, b.K(47.13)});
        aff(Vp37, {V, ONE, ZERO, ZERO, ZERO, ZERO, b.K(37.78)});
        aff(Vm10, {V, ONE, ZERO, ZERO, ZERO, ZERO, b.K(-10.0)});
        aff(LmL, {b.G(iCaL), MONE, ZERO, ZERO, ZERO, ZERO, b.K(p.LTRPNtot)});
        aff(HmH, {b.G(iCaH), MONE, ZERO, ZERO, ZERO, ZERO, b.K(p.HTRPNtot)});
        aff(KiNa02, {Ki, ONE, Nai, b.K(0.02), ZERO, ZERO, ZERO});
        if (!b.fast) {
            aff(argf, {L_Cai, b.K(p.Hf), ZERO, ZERO, ZERO, ZERO, b.K(-p.Hf * std::log(p.Kmf))});
            aff(argr, {L_NSR, b.K(p.Hr), ZERO, ZERO, ZERO, ZERO, b.K(-p.Hr * std::log(p.Kmr))});
        }
        b.warp_align(q);
        // 1 / (a0 + a1 a2 + a3 a4 + a5 a6 a7)
        auto rec = [&](uint16_t out, std::initializer_list<uint16_t> a) { b.emit(q, OK_REC, out, a); };
        rec(rKr, {ONE, b.K(1.4945), E_Kr});
        rec(rKp, {ONE, ONE, E_Kp});
        rec(rfNaK, {ONE, b.K(0.1245), E_e01, b.K(0.0365 * C.sigma), E_expm});
        rec(rNaCa, {ONE, b.K(p.ksat), E_e12});
        rec(r1me, {ONE, MONE, E_expm});
        rec(ram, {ONE, MONE, E_am});
        rec(rbh, {ONE, ONE, E_bh1});
        rec(raj, {ONE, ONE, E_aj3});
        rec(rbj, {ONE, ONE, E_bj2});
        rec(rxinf, {ONE, ONE, E_xinf});
        rec(rt1, {ONE, MONE, E_t1});
        rec(rt2, {MONE, ONE, E_t2});
        rec(rIpCa, {b.K(p.KmpCa), ONE, Cai});
        rec(rQ, {ZERO, ZERO, ZERO, ZERO, ZERO, Q23, Q34, ONE});
        rec(rC, {b.K(p.KCMDN), ONE, Cai});
        rec(rK1, {b.K(2.0), ZERO, ZERO, ZERO, ZERO, E_K1V, KiS, ONE});
        rec(rINaK, {b.K(std::pow(p.KmNai, 1.5)), ONE, NaS});
        rec(ry, {ONE, ONE, E_y});
        rec(rtau, {b.K(400.0), b.K(60.0), E_t});
        rec(JEXP, {ZERO, ZERO, ZERO, ZERO, ZERO, E_expm, E_expm, ONE});
        rec(rj, {ONE, ZERO, ZERO, ZERO, ZERO, MONE, E_expm, E_expm});
        b.warp_align(q);
        // LCC rate products of update_LCC_rates (GW_utils.tpp:118-186) at this V
        auto prod = [&](uint16_t out, std::initializer_list<uint16_t> a) { b.emit(q, OK_PROD, out, a); };
        const uint16_t c2 = b.KL(2.0), c3 = b.KL(3.0), c4 = b.KL(4.0), ca = b.K(C.a), cbi = b.K(C.binv);
        prod(A4, {c4, E_al});
        prod(A3, {c3, E_al});
        prod(A2, {c2, E_al});
        prod(B2, {c2, E_be});
        prod(B3, {c3, E_be});
        prod(B4, {c4, E_be});
        prod(A4a, {c4, E_al, ca});
        prod(A3a, {c3, E_al, ca});
        prod(A2a, {c2, E_al, ca});
        prod(A1a, {E_al, ca});
        prod(B1bi, {E_be, cbi});
        prod(B2bi, {c2, E_be, cbi});
        prod(B3bi, {c3, E_be, cbi});
        prod(B4bi, {c4, E_be, cbi});
        b.warp_align(q);
        if (b.fast) {
            b.emit(q, OK_SQRT, pf, {s1f, ONE, s1f, ONE});
            b.emit(q, OK_SQRT, pr, {s1r, ONE, s1r, ONE});
        }
    }
    // ---------------- phase C: PROD | REC | SUM | EXP ----------------
    {
        const int q = PH_C;
        auto prod = [&](uint16_t out, std::initializer_list<uint16_t> a) { b.emit(q, OK_PROD, out, a); };
        const uint16_t m = b.G(im), h = b.G(ih), Kr3 = b.G(iKr + 3);
        const double Kc = C.PKv14_Csc * kF * F_RT * 1.0e9;
        prod(T_INa, {b.K(p.GNa), m, m, m, h, b.G(ij), VmENa});
        prod(T_INab, {b.K(p.GNab), VmENa});
        prod(T_NaCa1, {b.K(C.INaCa_const * p.Cao), rNaCa, E_e1, Nai, Nai, Nai});
        prod(T_NaCa2, {b.K(C.INaCa_const * C.Nao3), rNaCa, E_e12, Cai});
        prod(P_NaK, {rfNaK, NaS, rINaK});
        prod(T_IKr, {b.K(p.GKr * C.sqrtKo * 0.5), rKr, Kr3, VmEK});
        prod(T_IKs, {b.K(p.GKs), b.G(ixKs), b.G(ixKs), VmEKs});
        prod(T_Kv14a, {b.K(Kc), V, b.G(iKv14 + 4), r1me, KiNa02});
        prod(T_Kv14b, {b.K(Kc * (p.Ko + 0.02 * p.Nao)), V, b.G(iKv14 + 4), r1me, E_expm});
        prod(T_Kv43, {b.K(p.GKv43), b.G(iKv43 + 4), VmEK});
        prod(P_Ito2a, {b.K(-C.Ito2_const * F_RT * p.Clcyto), V, r1me, E_expm});
        prod(P_Ito2b, {b.K(C.Ito2_const * F_RT * p.Clo), V, r1me});
        prod(T_IKp, {b.K(p.GKp), rKp, VmEK});
        prod(T_ICab, {b.K(p.GCab), VmECa});
        prod(T_IpCa, {b.K(p.IpCamax), rIpCa, Cai});
        prod(T_dL1, {b.K(p.kLTRPNp), Cai, LmL});
        prod(T_dL2, {b.K(p.kLTRPNm), b.G(iCaL)});
        prod(T_dH1, {b.K(p.kHTRPNp), Cai, HmH});
        prod(T_dH2, {b.K(p.kHTRPNm), b.G(iCaH)});
        const uint16_t c032 = b.K(0.32), c32 = b.K(3.2);
        if (r == 2)
            prod(T_am, {c32});
        else
            prod(T_am, {c032, ram, Vp47});
        prod(T_aj1, {raj, Vp37, E_aj1});
        prod(T_aj2, {raj, Vp37, E_aj2});
        prod(T_bj, {E_bj1, rbj});
        prod(T_t1, {b.K(0.0000719), Vm10, rt1});
        prod(T_t2, {b.K(0.000131), Vm10, rt2});
        prod(Q42, {Q32, Q43, Q24, rQ});
        prod(JMUL, {b.K(C.JLCC_const * F_RT), V, E_expm, E_expm, rj});
        b.warp_align(q);
        b.emit(q, OK_REC, beta, {ONE, ZERO, ZERO, ZERO, ZERO, b.K(C.CMDN_const), rC, rC});
        if (b.fast) b.emit(q, OK_REC, rJup, {ONE, ONE, pf, ONE, pr});
        b.warp_align(q);
        // yinf/tau = (0.4 ry + 0.6)(1 + E_t) rtau; (1 - yinf)/tau = (0.4 - 0.4 ry)(1 + E_t) rtau
        const uint16_t c04 = b.K(0.4), cm04 = b.K(-0.4), c06 = b.K(0.6);
        b.sum_row(q, INACT0, rtau, ONE, {{c04, ry, ONE}, {c04, ry, E_t}, {c06, ONE, ONE}, {c06, E_t, ONE}});
        b.sum_row(q, INACT1, rtau, ONE, {{c04, ONE, ONE}, {c04, E_t, ONE}, {cm04, ry, ONE}, {cm04, ry, E_t}});
        if (!b.fast) {
            b.warp_align(q);
            b.emit(q, OK_EXP, pf, {ONE, ONE, argf, ZERO});
            b.emit(q, OK_EXP, pr, {ONE, ONE, argr, ZERO});
        }
    }
    // ---------------- phase C2: general Jup exponents ----------------
    if (!b.fast) b.emit(PH_C2, OK_REC, rJup, {ONE, ONE, pf, ONE, pr});
    // ---------------- phase E: increments and update (OK_SUMU rows) ----------------
    b.post = false;
    b.upd_rows = true;
    {
        const int q = PH_E;
        using T = Builder::Term;
        const uint16_t DT = XS_DT;
        const double CSA = C.CSA_FVcyto;
        const uint16_t cGK1 = b.K(p.GK1 * C.IK1_const), cmGK1 = b.K(-p.GK1 * C.IK1_const);
        // dV (GW.tpp:211)
        b.sum_row(q, (uint16_t)(iV), DT, ONE,
                  {{ONE, XS_ISTIM, ONE}, {MONE, T_INa, ONE}, {b.K(-C.ICaL_const), SJLCC, ONE},
                   {MONE, T_IKr, ONE}, {MONE, T_IKs, ONE}, {MONE, T_Kv14a, ONE}, {ONE, T_Kv14b, ONE},
                   {MONE, T_Kv43, ONE}, {cmGK1, rK1, VmEK}, {MONE, T_IKp, ONE}, {MONE, P_Ito2a, SClCh},
                   {MONE, P_Ito2b, SClCh}, {b.K(-C.INaK_const), P_NaK, ONE}, {MONE, T_NaCa1, ONE},
                   {ONE, T_NaCa2, ONE}, {MONE, T_IpCa, ONE}, {MONE, T_ICab, ONE}, {MONE, T_INab, ONE}});
        const uint16_t cmCSA = b.K(-CSA);
        // dNai, dKi (GW.tpp:201-202)
        b.sum_row(q, (uint16_t)(iNai), DT, cmCSA,
                  {{ONE, T_INa, ONE}, {ONE, T_INab, ONE}, {b.K(3.0), T_NaCa1, ONE}, {b.K(-3.0), T_NaCa2, ONE},
                   {b.K(3.0 * C.INaK_const), P_NaK, ONE}});
        b.sum_row(q, (uint16_t)(iKi), DT, cmCSA,
                  {{ONE, T_IKr, ONE}, {ONE, T_IKs, ONE}, {ONE, T_Kv14a, ONE}, {MONE, T_Kv14b, ONE},
                   {ONE, T_Kv43, ONE}, {cGK1, rK1, VmEK}, {ONE, T_IKp, ONE}, {b.K(-2.0 * C.INaK_const), P_NaK, ONE}});
        // dCai, dCaNSR (GW.tpp:203-204)
        b.sum_row(q, (uint16_t)(iCai), DT, beta,
                  {{b.K(-0.5 * CSA), T_ICab, ONE}, {b.K(-0.5 * CSA), T_IpCa, ONE}, {b.K(CSA), T_NaCa1, ONE},
                   {b.K(-CSA), T_NaCa2, ONE}, {b.K(C.VSS_Vcyto * C.CRU_factor), SJxfer, ONE},
                   {b.K(-p.Vmaxf), rJup, pf}, {b.K(p.Vmaxr), rJup, pr}, {MONE, T_dL1, ONE}, {ONE, T_dL2, ONE},
                   {MONE, T_dH1, ONE}, {ONE, T_dH2, ONE}});
        b.sum_row(q, (uint16_t)(iCaNSR), DT, ONE,
                  {{b.K(C.Vcyto_VNSR * p.Vmaxf), rJup, pf}, {b.K(-C.Vcyto_VNSR * p.Vmaxr), rJup, pr},
                   {b.K(-C.VJSR_VNSR * C.CRU_factor), SJtr, ONE}});
        b.sum_row(q, (uint16_t)(iCaL), DT, ONE, {{ONE, T_dL1, ONE}, {MONE, T_dL2, ONE}});
        b.sum_row(q, (uint16_t)(iCaH), DT, ONE, {{ONE, T_dH1, ONE}, {MONE, T_dH2, ONE}});
        // gates (GW.tpp:163-168)
        b.sum_row(q, (uint16_t)(im), DT, ONE, {{ONE, T_am, ONE}, {MONE, T_am, b.G(im)}, {MONE, E_bm, b.G(im)}});
        const uint16_t cbh = b.K(-1.0 / 0.13);
        if (r0)
            b.sum_row(q, (uint16_t)(ih), DT, ONE, {{cbh, rbh, b.G(ih)}});
        else
            b.sum_row(q, (uint16_t)(ih), DT, ONE,
                      {{ONE, E_ah, ONE}, {MONE, E_ah, b.G(ih)}, {MONE, E_bh1, b.G(ih)}, {MONE, E_bh2, b.G(ih)}});
        b.sum_row(q, (uint16_t)(ij), DT, ONE,
                  {{ONE, T_aj1, ONE}, {ONE, T_aj2, ONE}, {MONE, T_aj1, b.G(ij)}, {MONE, T_aj2, b.G(ij)},
                   {MONE, T_bj, b.G(ij)}});
        b.sum_row(q, (uint16_t)(ixKs), DT, ONE,
                  {{ONE, T_t1, rxinf}, {ONE, T_t2, rxinf}, {MONE, T_t1, b.G(ixKs)}, {MONE, T_t2, b.G(ixKs)}});
        // IKr Markov chain (update_QKr + update_Kr_derivatives)
        const uint16_t cKf = b.K(p.Kf), cKb = b.K(p.Kb), cmKf = b.K(-p.Kf), cmKb = b.K(-p.Kb);
        auto kr = [&](int i) { return b.G(iKr + i); };
        b.sum_row(q, (uint16_t)(iKr + 0), DT, ONE, {{ONE, Q10, kr(1)}, {MONE, Q01, kr(0)}});
        b.sum_row(q, (uint16_t)(iKr + 1), DT, ONE, {{ONE, Q01, kr(0)}, {cKb, kr(2), ONE}, {MONE, Q10, kr(1)}, {cmKf, kr(1), ONE}});
        b.sum_row(q, (uint16_t)(iKr + 2), DT, ONE,
                  {{cKf, kr(1), ONE}, {ONE, Q32, kr(3)}, {ONE, Q42, kr(4)}, {cmKb, kr(2), ONE},
                   {MONE, Q23, kr(2)}, {MONE, Q24, kr(2)}});
        b.sum_row(q, (uint16_t)(iKr + 3), DT, ONE, {{ONE, Q23, kr(2)}, {ONE, Q43, kr(4)}, {MONE, Q32, kr(3)}, {MONE, Q34, kr(3)}});
        b.sum_row(q, (uint16_t)(iKr + 4), DT, ONE, {{ONE, Q24, kr(2)}, {ONE, Q34, kr(3)}, {MONE, Q42, kr(4)}, {MONE, Q43, kr(4)}});
        // Kv1.4 and Kv4.3 10-state chains (update_QKv + update_Kv_derivatives)
        for (int ch = 0; ch < 2; ++ch) {
            const int base = ch == 0 ? iKv14 : iKv43;
            const double f1 = ch == 0 ? p.f1Kv14 : p.f1Kv43, f2 = ch == 0 ? p.f2Kv14 : p.f2Kv43;
            const double f3 = ch == 0 ? p.f3Kv14 : p.f3Kv43, f4 = ch == 0 ? p.f4Kv14 : p.f4Kv43;
            const double b1 = ch == 0 ? p.b1Kv14 : p.b1Kv43, b2 = ch == 0 ? p.b2Kv14 : p.b2Kv43;
            const double b3 = ch == 0 ? p.b3Kv14 : p.b3Kv43, b4 = ch == 0 ? p.b4Kv14 : p.b4Kv43;
            const uint16_t aa = kv[ch][0], ai = kv[ch][1], ba = kv[ch][2], bi = kv[ch][3];
            auto x = [&](int i) { return b.G(base + i); };
            auto K = [&](double v) { return b.K(v); };
            auto L = [&](double v) { return b.KL(v); };
            b.sum_row(q, (uint16_t)(base + 0), DT, ONE, {{ONE, ba, x(1)}, {ONE, ai, x(5)}, {L(-4), aa, x(0)}, {MONE, bi, x(0)}});
            b.sum_row(q, (uint16_t)(base + 1), DT, ONE,
                      {{L(4), aa, x(0)}, {L(2), ba, x(2)}, {K(1 / b1), ai, x(6)}, {MONE, ba, x(1)}, {L(-3), aa, x(1)},
                       {K(-f1), bi, x(1)}});
            b.sum_row(q, (uint16_t)(base + 2), DT, ONE,
                      {{L(3), aa, x(1)}, {L(3), ba, x(3)}, {K(1 / b2), ai, x(7)}, {L(-2), ba, x(2)}, {L(-2), aa, x(2)},
                       {K(-f2), bi, x(2)}});
            b.sum_row(q, (uint16_t)(base + 3), DT, ONE,
                      {{L(2), aa, x(2)}, {L(4), ba, x(4)}, {K(1 / b3), ai, x(8)}, {L(-3), ba, x(3)}, {MONE, aa, x(3)},
                       {K(-f3), bi, x(3)}});
            b.sum_row(q, (uint16_t)(base + 4), DT, ONE, {{ONE, aa, x(3)}, {K(1 / b4), ai, x(9)}, {L(-4), ba, x(4)}, {K(-f4), bi, x(4)}});
            b.sum_row(q, (uint16_t)(base + 5), DT, ONE, {{K(1 / f1), ba, x(6)}, {ONE, bi, x(0)}, {K(-4 * b1), aa, x(5)}, {MONE, ai, x(5)}});
            b.sum_row(q, (uint16_t)(base + 6), DT, ONE,
                      {{K(4 * b1), aa, x(5)}, {K(2 * f1 / f2), ba, x(7)}, {K(f1), bi, x(1)}, {K(-1 / f1), ba, x(6)},
                       {K(-3 * b2 / b1), aa, x(6)}, {K(-1 / b1), ai, x(6)}});
            b.sum_row(q, (uint16_t)(base + 7), DT, ONE,
                      {{K(3 * b2 / b1), aa, x(6)}, {K(3 * f2 / f3), ba, x(8)}, {K(f2), bi, x(2)}, {K(-2 * f1 / f2), ba, x(7)},
                       {K(-2 * b3 / b2), aa, x(7)}, {K(-1 / b2), ai, x(7)}});
            b.sum_row(q, (uint16_t)(base + 8), DT, ONE,
                      {{K(2 * b3 / b2), aa, x(7)}, {K(4 * f3 / f4), ba, x(9)}, {K(f3), bi, x(3)}, {K(-3 * f2 / f3), ba, x(8)},
                       {K(-b4 / b3), aa, x(8)}, {K(-1 / b3), ai, x(8)}});
            b.sum_row(q, (uint16_t)(base + 9), DT, ONE,
                      {{K(b4 / b3), aa, x(8)}, {K(f4), bi, x(4)}, {K(-4 * f3 / f4), ba, x(9)}, {K(-1 / b4), ai, x(9)}});
        }
    }
    // per-step SSA values
    b.sv_src[SV_ZERO] = ZERO;
    b.sv_src[SV_A4] = A4; b.sv_src[SV_A3] = A3; b.sv_src[SV_A2] = A2; b.sv_src[SV_A1] = E_al;
    b.sv_src[SV_B1] = E_be; b.sv_src[SV_B2] = B2; b.sv_src[SV_B3] = B3; b.sv_src[SV_B4] = B4;
    b.sv_src[SV_A4a] = A4a; b.sv_src[SV_A3a] = A3a; b.sv_src[SV_A2a] = A2a; b.sv_src[SV_A1a] = A1a;
    b.sv_src[SV_B1bi] = B1bi; b.sv_src[SV_B2bi] = B2bi; b.sv_src[SV_B3bi] = B3bi; b.sv_src[SV_B4bi] = B4bi;
    b.sv_src[SV_F] = b.K(p.f); b.sv_src[SV_G] = b.K(p.g); b.sv_src[SV_OM] = b.K(C.omega);
    b.sv_src[SV_OMB1] = b.K(C.omega_b); b.sv_src[SV_OMB2] = b.K(C.omega_b2);
    b.sv_src[SV_OMB3] = b.K(C.omega_b3); b.sv_src[SV_OMB4] = b.K(C.omega_b4);
    b.sv_src[SV_F1] = b.K(p.f1); b.sv_src[SV_G1] = b.K(p.g1);
    b.sv_src[SV_INACT0] = INACT0; b.sv_src[SV_INACT1] = INACT1;
    b.sv_src[SV_JMUL] = JMUL; b.sv_src[SV_JEXP] = JEXP;
    b.sv_src[SV_CAI] = Cai; b.sv_src[SV_CANSR] = NSR;
    (void)argf;
    (void)argr;
}

int regime_of(double V, bool) { return V >= -40.0 ? 0 : (V == -47.13 ? 2 : 1); }

bool same_op(const OdeOp &a, const OdeOp &b) { return std::memcmp(&a, &b, sizeof a) == 0; }

}  // namespace

bool ode_program_build(const CellStatic &cs, bool pow_fast, OdeProgram *prog, double *consts) {
    Builder v[3] = {Builder(cs, pow_fast, 0, consts), Builder(cs, pow_fast, 1, nullptr),
                    Builder(cs, pow_fast, 2, nullptr)};
    for (auto &b : v) build(b);
    if (v[0].nconst > kOdeMaxConsts || v[0].next > kOdeMaxSlots) {
        if (prog) { prog->n_consts = v[0].nconst; prog->n_slots = v[0].next; }
        return false;
    }
    if (!prog) return true;
    std::memset(prog, 0, sizeof *prog);
    int n = 0;
    prog->n_phases = 0;
    for (int q = 0; q < PH_COUNT; ++q) {
        if (v[0].ph[q].empty()) continue;
        for (int k = 1; k < 3; ++k)
            if (v[k].ph[q].size() != v[0].ph[q].size()) {
                fprintf(stderr, "ode program: phase %d size differs in regime %d (%zu vs %zu)\n", q, k, v[k].ph[q].size(), v[0].ph[q].size());
                return false;
            }
        if (q == PH_E) prog->upd_phase = prog->n_phases;
        if (q == PH_C) prog->push_phase = prog->n_phases;
        prog->phase_begin[prog->n_phases++] = n;
        for (size_t j = 0; j < v[0].ph[q].size(); ++j) {
            if (n >= kOdeMaxOps) { fprintf(stderr, "ode program: too many ops\n"); return false; }
            prog->ops[n] = v[0].ph[q][j];
            prog->alt_idx[n] = 255;
            if (!same_op(v[1].ph[q][j], v[0].ph[q][j]) || !same_op(v[2].ph[q][j], v[0].ph[q][j])) {
                if (prog->n_alt >= kOdeMaxAlt) { fprintf(stderr, "ode program: too many variants\n"); return false; }
                prog->alt[0][prog->n_alt] = v[1].ph[q][j];
                prog->alt[1][prog->n_alt] = v[2].ph[q][j];
                prog->alt_idx[n] = (uint8_t)prog->n_alt++;
            }
            ++n;
        }
    }
    prog->phase_begin[prog->n_phases] = n;
    // Each warp of a phase must hold one op kind (in every regime): the device switches on it once
    // per warp.
    for (int q = 0; q < prog->n_phases; ++q) {
        const int b0 = prog->phase_begin[q], nq = prog->phase_begin[q + 1] - b0;
        if (nq > kOdeLanes) {
            fprintf(stderr, "ode program: phase %d has %d ops (max %d)\n", q, nq, kOdeLanes);
            return false;
        }
        for (int w = 0; w < kOdeWarps; ++w) {
            int kind = OK_NOP;
            for (int l = 32 * w; l < std::min(32 * w + 32, nq); ++l) {
                const OdeOp *cand[3] = {&prog->ops[b0 + l], nullptr, nullptr};
                if (prog->alt_idx[b0 + l] != 255) {
                    cand[1] = &prog->alt[0][prog->alt_idx[b0 + l]];
                    cand[2] = &prog->alt[1][prog->alt_idx[b0 + l]];
                }
                for (const OdeOp *op : cand) {
                    if (!op || op->kind == OK_NOP) continue;
                    if (kind != OK_NOP && kind != op->kind) {
                        fprintf(stderr, "ode program: phase %d warp %d mixes op kinds\n", q, w);
                        return false;
                    }
                    kind = op->kind;
                }
            }
            prog->wkind[q][w] = (uint8_t)kind;
        }
    }
    prog->n_slots = v[0].next;
    prog->const_begin = XS_FIRST_FREE;
    prog->n_consts = v[0].nconst;
    for (int i = 0; i < kSvCount; ++i) prog->sv_src[i] = v[0].sv_src[i];
    // The ops whose outputs are per-step SSA values stage them for the push themselves (Cai and
    // CaNSR are staged by their updates, constant values once per launch).
    for (int i = 0; i < kSvCount; ++i) {
        if (i == SV_CAI || i == SV_CANSR || i == SV_CAI_LO || i == SV_CANSR_LO) continue;
        const int src = prog->sv_src[i];
        if (src < XS_FIRST_FREE + kOdeMaxConsts) continue;  // fixed or constant slot
        for (int j = 0; j < n; ++j) {
            const bool writes = prog->ops[j].kind != OK_NOP && prog->ops[j].out == src;
            const bool alt_writes = prog->alt_idx[j] != 255 && (prog->alt[0][prog->alt_idx[j]].out == src ||
                                                                prog->alt[1][prog->alt_idx[j]].out == src);
            if (!writes && !alt_writes) continue;
            if (prog->sv_stage[j] != 0 && prog->sv_stage[j] != i + 1) {
                fprintf(stderr, "ode program: slot %d staged to two sv values\n", src);
                return false;
            }
            prog->sv_stage[j] = (uint8_t)(i + 1);
        }
    }
    return true;
}

// Host evaluation of one global step with the device's operation order (FP64): g[36] in/out,
// sums {JLCC, ClCh, Jtr, Jxfer}; sv receives the per-step SSA values of the updated state.
void ode_program_step_host(const OdeProgram &P, const double *consts, double *g, const double *sums,
                           double Istim, double dt, double *sv) {
    std::vector<double> X(kOdeMaxSlots, 0.0);
    X[XS_ZERO] = 0.0;
    X[XS_ONE] = 1.0;
    X[XS_MONE] = -1.0;
    for (int i = 0; i < P.n_consts; ++i) X[P.const_begin + i] = consts[i];
    for (int i = 0; i < kNumGlobals; ++i) X[XS_G + i] = X[XS_GN + i] = g[i];
    for (int i = 0; i < 4; ++i) X[XS_SUMS + i] = sums[i];
    X[XS_ISTIM] = Istim;
    X[XS_DT] = dt;
    auto regime = [&]() { const double V = g[0]; return V >= -40.0 ? 0 : (V == -47.13 ? 2 : 1); };
    auto run_phase = [&](int q, int reg) {
        const int b0 = P.phase_begin[q], n = P.phase_begin[q + 1] - b0;
        std::vector<double> val(n, 0.0);
        std::vector<const OdeOp *> ops(n);
        for (int j = 0; j < n; ++j) {
            const OdeOp *op = &P.ops[b0 + j];
            if (reg > 0 && P.alt_idx[b0 + j] != 255) op = &P.alt[reg - 1][P.alt_idx[b0 + j]];
            ops[j] = op;
            const uint16_t *a = op->a;
            double v = 0.0;
            switch (op->kind) {
            case OK_LOG: v = std::log(X[a[0]] + X[a[1]] * X[a[2]]); break;
            case OK_SQRT: v = X[a[0]] * X[a[1]] * std::sqrt(X[a[2]] * X[a[3]]); break;
            case OK_EXP: v = X[a[0]] * std::exp(X[a[1]] * X[a[2]] + X[a[3]]); break;
            case OK_AFF: v = X[a[0]] * X[a[1]] + X[a[2]] * X[a[3]] + X[a[4]] * X[a[5]] + X[a[6]]; break;
            case OK_REC: v = 1.0 / (X[a[0]] + X[a[1]] * X[a[2]] + X[a[3]] * X[a[4]] + X[a[5]] * X[a[6]] * X[a[7]]); break;
            case OK_PROD: v = X[a[0]] * X[a[1]] * X[a[2]] * X[a[3]] * X[a[4]] * X[a[5]] * X[a[6]]; break;
            case OK_SUM:
            case OK_SUMU:
                v = X[a[2]] * X[a[3]] * X[a[4]] + X[a[5]] * X[a[6]] * X[a[7]] + X[a[8]] * X[a[9]] * X[a[10]] +
                    X[a[11]] * X[a[12]] * X[a[13]];
                break;
            default: break;
            }
            val[j] = v;
        }
        // SUM rows: lane tree (offsets 1, 2, 4) as the device's shuffles, then the scale
        for (int off = 1; off < 8; off <<= 1)
            for (int j = 0; j < n; ++j)
                if ((ops[j]->kind == OK_SUM || ops[j]->kind == OK_SUMU) && (j % ops[j]->width) + off < ops[j]->width &&
                    (j % (2 * off)) == 0)
                    val[j] += val[j + off];
        for (int j = 0; j < n; ++j) {
            const OdeOp *op = ops[j];
            if (op->kind == OK_NOP) continue;
            if (op->kind == OK_SUMU) {
                // every row reads the old globals (XS_G) before any update, as on the device
                if (j % op->width == 0) {
                    g[op->out] += X[op->a[0]] * X[op->a[1]] * val[j];
                    X[XS_GN + op->out] = g[op->out];
                }
            } else if (op->kind == OK_SUM) {
                if (j % op->width == 0) X[op->out] = X[op->a[0]] * X[op->a[1]] * val[j];
            } else {
                X[op->out] = val[j];
            }
        }
    };
    // the transcendental phases of the current state (run before the loop on the device)
    for (int q = P.upd_phase + 1; q < P.n_phases; ++q) run_phase(q, regime());
    // the step: increments and update, then the new state's phases
    for (int q = 0; q < P.n_phases; ++q) run_phase(q, q <= P.upd_phase ? regime_of(g[0], true) : regime());
    for (int i = 0; i < kSvCount; ++i) sv[i] = X[P.sv_src[i]];
    for (int i = 0; i < kNumGlobals; ++i) X[XS_G + i] = X[XS_GN + i];
}

}  // namespace gw
