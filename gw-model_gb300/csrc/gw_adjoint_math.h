// gw_adjoint_math.h -- the continuous dynamics of one cell and their hand-written adjoints, for
// the pathwise gradients of gw_grad_* (gw_adjoint.cu).  Host and device.
//
// What is differentiated.  One global step of a cell (GW.tpp:237-272) is
//   G[s+1] = G[s] + d(G[s], carry[s], Istim[s]; theta)          (GW.tpp:26-212, 163-168, 127-160)
//   x[s+1] = Phi(x[s]; Cai[s], CaNSR[s], JM(V[s]), JE(V[s]); theta)    per CRU (SSA.tpp:286-310)
// where carry[s] = the flux sums the SSA of step s-1 left (sum JLCC, sum ClCh, sum Jtr, sum Jxfer;
// GW.tpp:188-198) and x = a CRU's continuous state (CaSS[4], CaJSR, JLCC[4]).  Conditional on the
// recorded jump trajectory (jump times, chosen transitions, binomial re-splits), Phi is a chain
// of explicit Euler sub-steps of CaSS and CaJSR (update_CaSS SSA.tpp:87-99, update_CaJSR
// SSA.hpp:68-71) whose lengths are the jump times, separated by events that reset JLCC
// (sample_LCC / sample_new_state, SSA.tpp:103-197, 262-283) or Jrel (sample_RyR, SSA.tpp:200-259).
// This pathwise estimator ignores the dependence of the jump times and of the chosen transitions
// on the parameters.  A binomial re-split of a lumped RyR pair changes no open count, so it has no
// effect on the continuous state.
//
// theta: the 8 parameters of the fit, each reported as a relative sensitivity theta_k dL/dtheta_k
//   PCaL (JLCC_const, through JLCC at LCC openings), GKr (IKr), GKs (IKs), GK1 (IK1),
//   INaKmax (INaK), Vmax (Vmaxf and Vmaxr scaled together: Jup), rRyR (Jrel), CSQNT (CaJSR buffer).
#pragma once

#include <cmath>

#include "gw_internal.h"

#ifdef __CUDACC__
#define GW_HD __host__ __device__ __forceinline__
#else
#define GW_HD inline
#endif

namespace gw {
namespace adj {

constexpr int kTheta = 8;
enum Theta { TH_PCAL = 0, TH_GKR = 1, TH_GKS = 2, TH_GK1 = 3, TH_INAK = 4, TH_VMAX = 5, TH_RRYR = 6, TH_CSQNT = 7 };
constexpr double kFaradayA = 96.5;  // common.hpp:9

// Flux sums of the previous step's SSA (the global step's inputs from the CRUs).
struct Carry {
    double jlcc, clch, jtr, jxfer;
};

GW_HD double sqd(double x) { return x * x; }
GW_HD double cubed(double x) { return x * x * x; }

// The transcendental terms of one global increment, each a function of the globals alone.  The
// increment and its adjoint read them from T[]; a block may evaluate them on kNT threads at once
// (on GB300 an FP64 instruction costs a sub-partition the same time for 1 or 32 active lanes) and
// pass them in: the values are the same bit for bit as one thread's.
enum Term {
    T_E = 0,    // exp(-V F/RT)
    T_LNA,      // log(Nao / Nai)
    T_LK,       // log(Ko / Ki)
    T_E1,       // exp(eta V F/RT)
    T_ENAK,     // exp(-0.1 V F/RT)
    T_PNAK,     // pow(KmNai / Nai, 1.5)
    T_RKR,      // exp(0.0446 V)
    T_LKS,      // log((Ko + 0.01833 Nao) / (Ki + 0.01833 Nai))
    T_K1,       // exp(1.5 (V - EK) F/RT)
    T_KP,       // exp((7.488 - V) / 5.98)
    T_FU,       // pow(Cai / Kmf, Hf)
    T_RU,       // pow(CaNSR / Kmr, Hr)
    T_AM,       // exp(-0.1 (V + 47.13))
    T_BM,       // exp(-V / 11)
    T_BH_HI,    // V >= -40: exp(-(V + 10.66) / 11.1)
    T_BJ_HI_Z,  //           exp(-0.1 (V + 32))
    T_BJ_HI_Y,  //           exp(-2.535e-7 V)
    T_AH_LO,    // V < -40:  exp(-(V + 80) / 6.8)
    T_BH_LO_1,  //           exp(0.079 V)
    T_BH_LO_2,  //           exp(0.35 V)
    T_AJ_A,     //           exp(0.2444 V)
    T_AJ_B,     //           exp(-0.04391 V)
    T_AJ_D,     //           exp(0.311 (V + 79.23))
    T_BJ_LO_Z,  //           exp(-0.1378 (V + 40.14))
    T_BJ_LO_Y,  //           exp(-0.01052 V)
    T_XINF,     // exp(-(V - 24.7) / 13.6)
    T_TAU1,     // exp(-0.148 (V - 10))
    T_TAU2,     // exp(0.0687 (V - 10))
    T_KR,       // 7 terms of the IKr chain: q01 q10 q23 q24 q32 q34 q43 without their prefactors
    T_KV14 = T_KR + 7,   // aa, ai, ba, bi of Kv1.4 without their prefactors
    T_KV43 = T_KV14 + 4,  // the same for Kv4.3
    kNT = T_KV43 + 4
};

GW_HD double glob_term(const CellStatic &C, const double *g, int k) {
    const gw_params &p = C.p;
    const double V = g[0];
    switch (k) {
    case T_E: return exp(-(V * C.F_RT));
    case T_LNA: return log(p.Nao / g[1]);
    case T_LK: return log(p.Ko / g[2]);
    case T_E1: return exp(p.eta * (V * C.F_RT));
    case T_ENAK: return exp(-0.1 * (V * C.F_RT));
    case T_PNAK: return pow(p.KmNai / g[1], 1.5);
    case T_RKR: return exp(0.0446 * V);
    case T_LKS: return log((p.Ko + 0.01833 * p.Nao) / (g[2] + 0.01833 * g[1]));
    case T_K1: {
        const double EK = log(p.Ko / g[2]) * C.RT_F / 1.0;
        return exp(1.5 * (V - EK) * C.F_RT);
    }
    case T_KP: return exp((7.488 - V) / 5.98);
    case T_FU: return pow(g[3] / p.Kmf, p.Hf);
    case T_RU: return pow(g[4] / p.Kmr, p.Hr);
    case T_AM: return exp(-0.1 * (V + 47.13));
    case T_BM: return exp(-V / 11.0);
    case T_BH_HI: return exp(-(V + 10.66) / 11.1);
    case T_BJ_HI_Z: return exp(-0.1 * (V + 32.0));
    case T_BJ_HI_Y: return exp(-2.535e-7 * V);
    case T_AH_LO: return exp(-(V + 80.0) / 6.8);
    case T_BH_LO_1: return exp(0.079 * V);
    case T_BH_LO_2: return exp(0.35 * V);
    case T_AJ_A: return exp(0.2444 * V);
    case T_AJ_B: return exp(-0.04391 * V);
    case T_AJ_D: return exp(0.311 * (V + 79.23));
    case T_BJ_LO_Z: return exp(-0.1378 * (V + 40.14));
    case T_BJ_LO_Y: return exp(-0.01052 * V);
    case T_XINF: return exp(-(V - 24.7) / 13.6);
    case T_TAU1: return exp(-0.148 * (V - 10.0));
    case T_TAU2: return exp(0.0687 * (V - 10.0));
    case T_KR + 0: return exp(0.0272 * V);
    case T_KR + 1: return exp(-0.0431 * V);
    case T_KR + 2: return exp(0.0262 * V);
    case T_KR + 3: return exp(2.71e-6 * V);
    case T_KR + 4: return exp(-0.0269 * V);
    case T_KR + 5: return exp(0.0120 * V);
    case T_KR + 6: return exp(-0.0443 * V);
    case T_KV14 + 0: return exp(p.aaKv14 * V);
    case T_KV14 + 1: return exp(-p.aiKv14 * V);
    case T_KV14 + 2: return exp(-p.baKv14 * V);
    case T_KV14 + 3: return exp(p.biKv14 * V);
    case T_KV43 + 0: return exp(p.aaKv43 * V);
    case T_KV43 + 1: return exp(-p.aiKv43 * V);
    case T_KV43 + 2: return exp(-p.baKv43 * V);
    case T_KV43 + 3: return exp(p.biKv43 * V);
    default: return 0.0;
    }
}

GW_HD void glob_terms(const CellStatic &C, const double *g, double *T) {
    for (int k = 0; k < kNT; ++k) T[k] = glob_term(C, g, k);
}

// ---------------------------------------------------------------------------------------------
// The global increment d = G[s+1] - G[s] (update_V_and_concentration_derivatives GW.tpp:171-212,
// update_gate_derivatives :163-168, update_Kr/Kv_derivatives :127-160 with update_QKr/QKv
// :26-123), in the reference's formulas and operation order.
// ---------------------------------------------------------------------------------------------

// Rates of the Kv1.4 / Kv4.3 chains (update_QKv, GW.tpp:65-123): aa, ai, ba, bi.
GW_HD void kv_rates(const gw_params &p, int ch, const double *T, double r[4]) {
    if (ch == 0) {
        r[0] = p.alphaa0Kv14 * T[T_KV14 + 0];
        r[1] = p.alphai0Kv14 * T[T_KV14 + 1];
        r[2] = p.betaa0Kv14 * T[T_KV14 + 2];
        r[3] = p.betai0Kv14 * T[T_KV14 + 3];
    } else {
        r[0] = p.alphaa0Kv43 * T[T_KV43 + 0];
        r[1] = p.alphai0Kv43 * T[T_KV43 + 1];
        r[2] = p.betaa0Kv43 * T[T_KV43 + 2];
        r[3] = p.betai0Kv43 * T[T_KV43 + 3];
    }
}

// The off-diagonal transitions of a 10-state Kv chain: from, to, coefficient, rate (0 aa, 1 ai,
// 2 ba, 3 bi), as update_QKv builds them; the diagonal is minus the row sum.
struct KvEdge {
    int a, b;
    double coef;
    int rate;
};
GW_HD void kv_edges(const gw_params &p, int ch, KvEdge e[26]) {
    const double f1 = ch == 0 ? p.f1Kv14 : p.f1Kv43, f2 = ch == 0 ? p.f2Kv14 : p.f2Kv43;
    const double f3 = ch == 0 ? p.f3Kv14 : p.f3Kv43, f4 = ch == 0 ? p.f4Kv14 : p.f4Kv43;
    const double b1 = ch == 0 ? p.b1Kv14 : p.b1Kv43, b2 = ch == 0 ? p.b2Kv14 : p.b2Kv43;
    const double b3 = ch == 0 ? p.b3Kv14 : p.b3Kv43, b4 = ch == 0 ? p.b4Kv14 : p.b4Kv43;
    int n = 0;
    auto E = [&](int a, int b, double c, int r) { e[n++] = KvEdge{a, b, c, r}; };
    E(0, 1, 4.0, 0); E(0, 5, 1.0, 3);
    E(1, 0, 1.0, 2); E(1, 2, 3.0, 0); E(1, 6, f1, 3);
    E(2, 1, 2.0, 2); E(2, 3, 2.0, 0); E(2, 7, f2, 3);
    E(3, 2, 3.0, 2); E(3, 4, 1.0, 0); E(3, 8, f3, 3);
    E(4, 3, 4.0, 2); E(4, 9, f4, 3);
    E(5, 6, 4.0 * b1, 0); E(5, 0, 1.0, 1);
    E(6, 5, 1.0 / f1, 2); E(6, 7, 3.0 * b2 / b1, 0); E(6, 1, 1.0 / b1, 1);
    E(7, 6, 2.0 * f1 / f2, 2); E(7, 8, 2.0 * b3 / b2, 0); E(7, 2, 1.0 / b2, 1);
    E(8, 7, 3.0 * f2 / f3, 2); E(8, 9, b4 / b3, 0); E(8, 3, 1.0 / b3, 1);
    E(9, 8, 4.0 * f3 / f4, 2); E(9, 4, 1.0 / b4, 1);
}

// Q matrix of one Kv chain in the reference's arithmetic (fill order of update_QKv).
GW_HD void kv_matrix(const gw_params &p, int ch, const double *T, double Q[10][10]) {
    double r[4];
    kv_rates(p, ch, T, r);
    const double aa = r[0], ai = r[1], ba = r[2], bi = r[3];
    const double f1 = ch == 0 ? p.f1Kv14 : p.f1Kv43, f2 = ch == 0 ? p.f2Kv14 : p.f2Kv43;
    const double f3 = ch == 0 ? p.f3Kv14 : p.f3Kv43, f4 = ch == 0 ? p.f4Kv14 : p.f4Kv43;
    const double b1 = ch == 0 ? p.b1Kv14 : p.b1Kv43, b2 = ch == 0 ? p.b2Kv14 : p.b2Kv43;
    const double b3 = ch == 0 ? p.b3Kv14 : p.b3Kv43, b4 = ch == 0 ? p.b4Kv14 : p.b4Kv43;
    Q[0][1] = 4 * aa; Q[0][5] = bi; Q[0][0] = -(Q[0][1] + Q[0][5]);
    Q[1][0] = ba; Q[1][2] = 3 * aa; Q[1][6] = f1 * bi; Q[1][1] = -(Q[1][0] + Q[1][2] + Q[1][6]);
    Q[2][1] = 2 * ba; Q[2][3] = 2 * aa; Q[2][7] = f2 * bi; Q[2][2] = -(Q[2][1] + Q[2][3] + Q[2][7]);
    Q[3][2] = 3 * ba; Q[3][4] = aa; Q[3][8] = f3 * bi; Q[3][3] = -(Q[3][2] + Q[3][4] + Q[3][8]);
    Q[4][3] = 4 * ba; Q[4][9] = f4 * bi; Q[4][4] = -(Q[4][3] + Q[4][9]);
    Q[5][6] = 4 * aa * b1; Q[5][0] = ai; Q[5][5] = -(Q[5][6] + Q[5][0]);
    Q[6][5] = ba / f1; Q[6][7] = 3 * aa * b2 / b1; Q[6][1] = ai / b1;
    Q[6][6] = -(Q[6][5] + Q[6][7] + Q[6][1]);
    Q[7][6] = 2 * ba * f1 / f2; Q[7][8] = 2 * aa * b3 / b2; Q[7][2] = ai / b2;
    Q[7][7] = -(Q[7][6] + Q[7][8] + Q[7][2]);
    Q[8][7] = 3 * ba * f2 / f3; Q[8][9] = aa * b4 / b3; Q[8][3] = ai / b3;
    Q[8][8] = -(Q[8][7] + Q[8][9] + Q[8][3]);
    Q[9][8] = 4 * ba * f3 / f4; Q[9][4] = ai / b4; Q[9][9] = -(Q[9][8] + Q[9][4]);
}

// Stencil of update_Kv_derivatives (GW.tpp:136-160): d = dt * (incoming + diagonal) per state.
GW_HD void kv_deriv(const double Q[10][10], const double *x, double *d, double dt) {
    d[0] = dt * (Q[1][0] * x[1] + Q[5][0] * x[5] + Q[0][0] * x[0]);
    d[1] = dt * (Q[0][1] * x[0] + Q[2][1] * x[2] + Q[6][1] * x[6] + Q[1][1] * x[1]);
    d[2] = dt * (Q[1][2] * x[1] + Q[3][2] * x[3] + Q[7][2] * x[7] + Q[2][2] * x[2]);
    d[3] = dt * (Q[2][3] * x[2] + Q[4][3] * x[4] + Q[8][3] * x[8] + Q[3][3] * x[3]);
    d[4] = dt * (Q[3][4] * x[3] + Q[9][4] * x[9] + Q[4][4] * x[4]);
    d[5] = dt * (Q[6][5] * x[6] + Q[0][5] * x[0] + Q[5][5] * x[5]);
    d[6] = dt * (Q[5][6] * x[5] + Q[7][6] * x[7] + Q[1][6] * x[1] + Q[6][6] * x[6]);
    d[7] = dt * (Q[6][7] * x[6] + Q[8][7] * x[8] + Q[2][7] * x[2] + Q[7][7] * x[7]);
    d[8] = dt * (Q[7][8] * x[7] + Q[9][8] * x[9] + Q[3][8] * x[3] + Q[8][8] * x[8]);
    d[9] = dt * (Q[8][9] * x[8] + Q[4][9] * x[4] + Q[9][9] * x[9]);
}

// IKr chain (update_QKr, GW.tpp:26-44): the V-dependent entries Q01 Q10 Q23 Q24 Q32 Q34 Q43 and
// Q42 = Q32 Q43 Q24 / (Q23 Q34).
struct KrQ {
    double q01, q10, q23, q24, q32, q34, q43, q42;
};
GW_HD KrQ kr_q(const double *T) {
    KrQ q;
    q.q01 = 0.0069 * T[T_KR + 0];
    q.q10 = 0.0227 * T[T_KR + 1];
    q.q23 = 0.0218 * T[T_KR + 2];
    q.q24 = 1.29e-5 * T[T_KR + 3];
    q.q32 = 0.0009 * T[T_KR + 4];
    q.q34 = 0.0622 * T[T_KR + 5];
    q.q43 = 0.0059 * T[T_KR + 6];
    q.q42 = q.q32 * q.q43 * q.q24 / (q.q23 * q.q34);
    return q;
}

// The gate rate functions of update_gate_derivatives (common.hpp:175-218, GW_utils.hpp:358-362)
// and their V derivatives.  The h and j rates change form at V = -40 mV (a discontinuity of the
// reference's model).
struct Gates {
    double am, bm, ah, bh, aj, bj, xinf, tinv;
    double dam, dbm, dah, dbh, daj, dbj, dxinf, dtinv;
};
GW_HD Gates gate_rates(double V, bool derivs, const double *T) {
    Gates r{};
    const bool hi = V >= -40.0;
    {
        const double w = V + 47.13, E = T[T_AM];
        r.am = (V == -47.13) ? 3.2 : 0.32 * w / (1.0 - E);
        if (derivs) r.dam = (V == -47.13) ? 0.16 : 0.32 * ((1.0 - E) - w * 0.1 * E) / sqd(1.0 - E);
    }
    r.bm = 0.08 * T[T_BM];
    r.dbm = -r.bm / 11.0;
    if (hi) {
        r.ah = 0.0;
        const double X = T[T_BH_HI];
        r.bh = 1.0 / (0.13 * (1.0 + X));
        r.dbh = r.bh * X / (11.1 * (1.0 + X));
        r.aj = 0.0;
        const double Z = T[T_BJ_HI_Z], y0 = 0.3 * T[T_BJ_HI_Y];
        r.bj = y0 / (1.0 + Z);
        r.dbj = r.bj * (-2.535e-7 + 0.1 * Z / (1.0 + Z));
    } else {
        r.ah = 0.135 * T[T_AH_LO];
        r.dah = -r.ah / 6.8;
        const double e1 = T[T_BH_LO_1], e2 = T[T_BH_LO_2];
        r.bh = 3.56 * e1 + 3.1e5 * e2;
        r.dbh = 3.56 * 0.079 * e1 + 3.1e5 * 0.35 * e2;
        const double ea = T[T_AJ_A], eb = T[T_AJ_B];
        const double P = -127140.0 * ea - 3.474e-5 * eb, Qv = V + 37.78;
        const double D = 1.0 + T[T_AJ_D];
        r.aj = P * Qv / D;
        const double dP = -127140.0 * 0.2444 * ea + 3.474e-5 * 0.04391 * eb, dD = 0.311 * (D - 1.0);
        r.daj = (dP * Qv + P) / D - P * Qv * dD / sqd(D);
        const double Z = T[T_BJ_LO_Z], y0 = 0.1212 * T[T_BJ_LO_Y];
        r.bj = y0 / (1.0 + Z);
        r.dbj = r.bj * (-0.01052 + 0.1378 * Z / (1.0 + Z));
    }
    {
        const double X = T[T_XINF];
        r.xinf = 1.0 / (1.0 + X);
        r.dxinf = r.xinf * r.xinf * X / 13.6;
    }
    {
        const double u = V - 10.0, E1 = T[T_TAU1], E2 = T[T_TAU2];
        r.tinv = 0.0000719 * u / (1.0 - E1) + 0.000131 * u / (E2 - 1.0);
        r.dtinv = 0.0000719 * ((1.0 - E1) - u * 0.148 * E1) / sqd(1.0 - E1) +
                  0.000131 * ((E2 - 1.0) - u * 0.0687 * E2) / sqd(E2 - 1.0);
    }
    return r;
}

// The global increment (the same formulas and order as the reference) in three dependency levels,
// so that a block can evaluate each level's items one per thread:
//   glob_term   (level 1) the transcendental terms T, functions of the globals alone;
//   kv_entry    (level 2) the off-diagonal Kv generator entries, functions of T;
//   glob_qty    (level 3) the currents, fluxes and buffer factors, and the derivative components
//               d[7..35] of the gates and Markov chains, functions of the globals, T, the carry and
//               the Kv entries;
//   glob_dconc  (level 4) d[0..6], linear combinations of the level-3 currents.
// glob_increment runs the levels one item after the other; the values are the same either way.

// Off-diagonal entries of the Kv4.3 (channel 1) and Kv1.4 (channel 0) generators, in the fill order
// of update_QKv (GW.tpp:65-123): entry e < 26 of channel ch is kv_edges' edge e.
constexpr int kKvE = 26;
GW_HD double kv_entry(const gw_params &p, const double *T, int k) {
    const int ch = k < kKvE ? 1 : 0, e = k % kKvE;
    double r[4];
    kv_rates(p, ch, T, r);
    const double aa = r[0], ai = r[1], ba = r[2], bi = r[3];
    const double f1 = ch == 0 ? p.f1Kv14 : p.f1Kv43, f2 = ch == 0 ? p.f2Kv14 : p.f2Kv43;
    const double f3 = ch == 0 ? p.f3Kv14 : p.f3Kv43, f4 = ch == 0 ? p.f4Kv14 : p.f4Kv43;
    const double b1 = ch == 0 ? p.b1Kv14 : p.b1Kv43, b2 = ch == 0 ? p.b2Kv14 : p.b2Kv43;
    const double b3 = ch == 0 ? p.b3Kv14 : p.b3Kv43, b4 = ch == 0 ? p.b4Kv14 : p.b4Kv43;
    switch (e) {
    case 0: return 4 * aa;          // Q01
    case 1: return bi;              // Q05
    case 2: return ba;              // Q10
    case 3: return 3 * aa;          // Q12
    case 4: return f1 * bi;         // Q16
    case 5: return 2 * ba;          // Q21
    case 6: return 2 * aa;          // Q23
    case 7: return f2 * bi;         // Q27
    case 8: return 3 * ba;          // Q32
    case 9: return aa;              // Q34
    case 10: return f3 * bi;        // Q38
    case 11: return 4 * ba;         // Q43
    case 12: return f4 * bi;        // Q49
    case 13: return 4 * aa * b1;    // Q56
    case 14: return ai;             // Q50
    case 15: return ba / f1;        // Q65
    case 16: return 3 * aa * b2 / b1;  // Q67
    case 17: return ai / b1;        // Q61
    case 18: return 2 * ba * f1 / f2;  // Q76
    case 19: return 2 * aa * b3 / b2;  // Q78
    case 20: return ai / b2;        // Q72
    case 21: return 3 * ba * f2 / f3;  // Q87
    case 22: return aa * b4 / b3;   // Q89
    case 23: return ai / b3;        // Q83
    case 24: return 4 * ba * f3 / f4;  // Q98
    default: return ai / b4;        // Q94
    }
}

// The Q matrix of a channel from its entries E[26] (the diagonal as update_QKv forms it).
GW_HD void kv_fill(const double *E, double Q[10][10]) {
    Q[0][1] = E[0]; Q[0][5] = E[1]; Q[0][0] = -(Q[0][1] + Q[0][5]);
    Q[1][0] = E[2]; Q[1][2] = E[3]; Q[1][6] = E[4]; Q[1][1] = -(Q[1][0] + Q[1][2] + Q[1][6]);
    Q[2][1] = E[5]; Q[2][3] = E[6]; Q[2][7] = E[7]; Q[2][2] = -(Q[2][1] + Q[2][3] + Q[2][7]);
    Q[3][2] = E[8]; Q[3][4] = E[9]; Q[3][8] = E[10]; Q[3][3] = -(Q[3][2] + Q[3][4] + Q[3][8]);
    Q[4][3] = E[11]; Q[4][9] = E[12]; Q[4][4] = -(Q[4][3] + Q[4][9]);
    Q[5][6] = E[13]; Q[5][0] = E[14]; Q[5][5] = -(Q[5][6] + Q[5][0]);
    Q[6][5] = E[15]; Q[6][7] = E[16]; Q[6][1] = E[17]; Q[6][6] = -(Q[6][5] + Q[6][7] + Q[6][1]);
    Q[7][6] = E[18]; Q[7][8] = E[19]; Q[7][2] = E[20]; Q[7][7] = -(Q[7][6] + Q[7][8] + Q[7][2]);
    Q[8][7] = E[21]; Q[8][9] = E[22]; Q[8][3] = E[23]; Q[8][8] = -(Q[8][7] + Q[8][9] + Q[8][3]);
    Q[9][8] = E[24]; Q[9][4] = E[25]; Q[9][9] = -(Q[9][8] + Q[9][4]);
}

// Component i of update_Kv_derivatives (GW.tpp:136-160) from the channel's entries E[26].
GW_HD double kv_component(const double *E, const double *x, int i, double dt) {
    double Q[10][10];
    kv_fill(E, Q);
    switch (i) {
    case 0: return dt * (Q[1][0] * x[1] + Q[5][0] * x[5] + Q[0][0] * x[0]);
    case 1: return dt * (Q[0][1] * x[0] + Q[2][1] * x[2] + Q[6][1] * x[6] + Q[1][1] * x[1]);
    case 2: return dt * (Q[1][2] * x[1] + Q[3][2] * x[3] + Q[7][2] * x[7] + Q[2][2] * x[2]);
    case 3: return dt * (Q[2][3] * x[2] + Q[4][3] * x[4] + Q[8][3] * x[8] + Q[3][3] * x[3]);
    case 4: return dt * (Q[3][4] * x[3] + Q[9][4] * x[9] + Q[4][4] * x[4]);
    case 5: return dt * (Q[6][5] * x[6] + Q[0][5] * x[0] + Q[5][5] * x[5]);
    case 6: return dt * (Q[5][6] * x[5] + Q[7][6] * x[7] + Q[1][6] * x[1] + Q[6][6] * x[6]);
    case 7: return dt * (Q[6][7] * x[6] + Q[8][7] * x[8] + Q[2][7] * x[2] + Q[7][7] * x[7]);
    case 8: return dt * (Q[7][8] * x[7] + Q[9][8] * x[9] + Q[3][8] * x[3] + Q[8][8] * x[8]);
    default: return dt * (Q[8][9] * x[8] + Q[4][9] * x[4] + Q[9][9] * x[9]);
    }
}

// Level-3 quantities.
enum Qty {
    Q_INA = 0, Q_INAB, Q_INACA, Q_INAK, Q_IKR, Q_IKS, Q_IKV14, Q_IKV43, Q_ITO2, Q_IK1, Q_IKP, Q_ICAL, Q_ICAB,
    Q_IPCA, Q_JUP, Q_BETA, Q_DLT, Q_DHT,
    Q_D,              // d[7 + i], i = 0 .. 28: gates m h j xKs, IKr chain, Kv4.3, Kv1.4
    kNQ = Q_D + 29
};

GW_HD double glob_qty(const CellStatic &C, const double *g, const Carry &cy, double dt, const double *T,
                      const double *KvE, int k) {
    const gw_params &p = C.p;
    const double V = g[0], Nai = g[1], Ki = g[2], Cai = g[3], CaNSR = g[4], CaLT = g[5], CaHT = g[6];
    const double m = g[7], h = g[8], jg = g[9], xKs = g[10];
    const double *Kr = g + 11, *Kv43 = g + 16, *Kv14 = g + 26;
    const double VF_RT = V * C.F_RT, e = T[T_E];
    const double ENa = T[T_LNA] * C.RT_F / 1.0;
    const double EK = T[T_LK] * C.RT_F / 1.0;
    const double ECa = T[T_LK] * C.RT_F / 2.0;
    (void)CaNSR;
    switch (k) {
    case Q_INA: return p.GNa * cubed(m) * h * jg * (V - ENa);
    case Q_INAB: return p.GNab * (V - ENa);
    case Q_INACA: {
        const double e1 = T[T_E1], e2 = e1 * e;
        return C.INaCa_const * (e1 * cubed(Nai) * p.Cao - e2 * C.Nao3 * Cai) / (1.0 + p.ksat * e2);
    }
    case Q_INAK: {
        const double fNaK = 1.0 / (1.0 + 0.1245 * T[T_ENAK] + 0.0365 * C.sigma * e);
        return C.INaK_const * fNaK / (1.0 + T[T_PNAK]);
    }
    case Q_IKR: {
        const double RKr = 1.0 / (1.0 + 1.4945 * T[T_RKR]);
        return p.GKr * C.sqrtKo * RKr * Kr[3] * (V - EK) * 0.5;
    }
    case Q_IKS: return p.GKs * sqd(xKs) * (V - T[T_LKS] * C.RT_F);
    case Q_IKV14: {
        const double mm = C.PKv14_Csc * (kFaradayA * VF_RT) * Kv14[4] / (1 - e);
        return mm * ((Ki - p.Ko * e) + 0.02 * (Nai - p.Nao * e)) * 1.0e9;
    }
    case Q_IKV43: return p.GKv43 * Kv43[4] * (V - EK);
    case Q_ITO2: return cy.clch * C.Ito2_const * VF_RT * (p.Clcyto * e - p.Clo) / (e - 1.0);
    case Q_IK1: return p.GK1 * (1.0 / (2.0 + T[T_K1])) * C.IK1_const * (V - EK);
    case Q_IKP: return p.GKp * (1. / (1. + T[T_KP])) * (V - EK);
    case Q_ICAL: return cy.jlcc * C.ICaL_const;
    case Q_ICAB: return p.GCab * (V - ECa);
    case Q_IPCA: return p.IpCamax * (Cai / (p.KmpCa + Cai));
    case Q_JUP: {
        const double fu = T[T_FU], ru = T[T_RU];
        return (p.Vmaxf * fu - p.Vmaxr * ru) / (1.0 + fu + ru);
    }
    case Q_BETA: return 1.0 / (1.0 + C.CMDN_const / sqd(p.KCMDN + Cai));
    case Q_DLT: return p.kLTRPNp * Cai * (p.LTRPNtot - CaLT) - p.kLTRPNm * CaLT;
    case Q_DHT: return p.kHTRPNp * Cai * (p.HTRPNtot - CaHT) - p.kHTRPNm * CaHT;
    default: break;
    }
    const int i = k - Q_D;
    if (i < 4) {
        const Gates gr = gate_rates(V, false, T);
        switch (i) {
        case 0: return dt * (gr.am * (1.0 - m) - gr.bm * m);
        case 1: return dt * (gr.ah * (1.0 - h) - gr.bh * h);
        case 2: return dt * (gr.aj * (1.0 - jg) - gr.bj * jg);
        default: return dt * (gr.xinf - xKs) * gr.tinv;
        }
    }
    if (i < 9) {
        const KrQ q = kr_q(T);
        switch (i - 4) {
        case 0: return dt * (q.q10 * Kr[1] + (-q.q01) * Kr[0]);
        case 1: return dt * (q.q01 * Kr[0] + p.Kb * Kr[2] + (-(q.q10 + p.Kf)) * Kr[1]);
        case 2: return dt * (p.Kf * Kr[1] + q.q32 * Kr[3] + q.q42 * Kr[4] + (-(p.Kb + q.q23 + q.q24)) * Kr[2]);
        case 3: return dt * (q.q23 * Kr[2] + q.q43 * Kr[4] + (-(q.q32 + q.q34)) * Kr[3]);
        default: return dt * (q.q24 * Kr[2] + q.q34 * Kr[3] + (-(q.q42 + q.q43)) * Kr[4]);
        }
    }
    if (i < 19) return kv_component(KvE, Kv43, i - 9, dt);
    return kv_component(KvE + kKvE, Kv14, i - 19, dt);
}

// d[k], k < 7, from the level-3 quantities Qv.
GW_HD double glob_dconc(const CellStatic &C, const Carry &cy, double Istim, double dt, const double *Qv, int k) {
    const double INa = Qv[Q_INA], INab = Qv[Q_INAB], INaCa = Qv[Q_INACA], INaK = Qv[Q_INAK];
    const double IKr = Qv[Q_IKR], IKs = Qv[Q_IKS], Ito1 = Qv[Q_IKV14] + Qv[Q_IKV43], IK1 = Qv[Q_IK1];
    const double IKp = Qv[Q_IKP];
    switch (k) {
    case 0:
        return dt * (Istim - (INa + Qv[Q_ICAL] + IKr + IKs + Ito1 + IK1 + IKp + Qv[Q_ITO2] + INaK + INaCa +
                              Qv[Q_IPCA] + Qv[Q_ICAB] + INab));
    case 1: return -dt * C.CSA_FVcyto * (INa + INab + 3 * INaCa + 3 * INaK);
    case 2: return -dt * C.CSA_FVcyto * (IKr + IKs + Ito1 + IK1 + IKp - 2 * INaK);
    case 3:
        return dt * Qv[Q_BETA] *
               (-0.5 * C.CSA_FVcyto * (Qv[Q_ICAB] + Qv[Q_IPCA] - 2 * INaCa) + C.VSS_Vcyto * (cy.jxfer * C.CRU_factor) -
                Qv[Q_JUP] - (Qv[Q_DLT] + Qv[Q_DHT]));
    case 4: return dt * (C.Vcyto_VNSR * Qv[Q_JUP] - C.VJSR_VNSR * (cy.jtr * C.CRU_factor));
    case 5: return Qv[Q_DLT] * dt;
    default: return Qv[Q_DHT] * dt;
    }
}

// The global increment d = G[s+1] - G[s] from the globals g and their terms T.  Returns false for a
// non-positive Nernst argument, where the reference exits (common.hpp:72-75).
GW_HD bool glob_increment(const CellStatic &C, const double *g, const Carry &cy, double Istim, double dt,
                          const double *T, double *d) {
    if (!(g[1] > 0.0) || !(g[2] > 0.0)) return false;
    double E[2 * kKvE], Qv[kNQ];
    for (int k = 0; k < 2 * kKvE; ++k) E[k] = kv_entry(C.p, T, k);
    for (int k = 0; k < kNQ; ++k) Qv[k] = glob_qty(C, g, cy, dt, T, E, k);
    for (int k = 0; k < 7; ++k) d[k] = glob_dconc(C, cy, Istim, dt, Qv, k);
    for (int k = 0; k < 29; ++k) d[7 + k] = Qv[Q_D + k];
    return true;
}

// Per-step SSA values of a state (the lane's sv[], gw_internal.h SvIndex) in the reference's
// arithmetic: update_LCC_rates (GW_utils.tpp:118-186), update_LCC_inactivation_rates
// (GW_utils.hpp:378-383) and the JLCC factors (GW.tpp:216-221).
// Their transcendental terms, by index (as glob_term).
enum SvTerm { S_E = 0, S_AL, S_BE, S_Y, S_TAU, kNS };
GW_HD double sv_term(const CellStatic &C, const double *g, int k) {
    const double V = g[0];
    switch (k) {
    case S_E: return exp(-(V * C.F_RT));
    case S_AL: return exp(0.012 * (V - 35.0));
    case S_BE: return exp(-0.05 * (V - 35.0));
    case S_Y: return exp((V + 12.5) / 5.0);
    default: return exp((V + 30.0) / 12.0);
    }
}
GW_HD void step_values(const CellStatic &C, const double *g, const double *S, double *sv) {
    const double V = g[0];
    const double e = S[S_E];
    const double al = 2.0 * S[S_AL];
    const double be = 0.0882 * S[S_BE];
    const double yinf = 0.4 / (1.0 + S[S_Y]) + 0.6;
    const double tau = 340.0 / (1.0 + S[S_TAU]) + 60.0;
    const double JE = sqd(1.0 / e);
    for (int i = 0; i < kSvCount; ++i) sv[i] = 0.0;
    sv[SV_A4] = 4 * al; sv[SV_A3] = 3 * al; sv[SV_A2] = 2 * al; sv[SV_A1] = al;
    sv[SV_B1] = be; sv[SV_B2] = 2 * be; sv[SV_B3] = 3 * be; sv[SV_B4] = 4 * be;
    sv[SV_A4a] = 4 * al * C.a; sv[SV_A3a] = 3 * al * C.a; sv[SV_A2a] = 2 * al * C.a; sv[SV_A1a] = al * C.a;
    sv[SV_B1bi] = be * C.binv; sv[SV_B2bi] = 2 * be * C.binv; sv[SV_B3bi] = 3 * be * C.binv;
    sv[SV_B4bi] = 4 * be * C.binv;
    sv[SV_F] = C.p.f; sv[SV_G] = C.p.g; sv[SV_OM] = C.omega;
    sv[SV_OMB1] = C.omega_b; sv[SV_OMB2] = C.omega_b2; sv[SV_OMB3] = C.omega_b3; sv[SV_OMB4] = C.omega_b4;
    sv[SV_F1] = C.p.f1; sv[SV_G1] = C.p.g1;
    sv[SV_INACT0] = yinf / tau;
    sv[SV_INACT1] = (1.0 - yinf) / tau;
    sv[SV_JEXP] = JE;
    sv[SV_JMUL] = C.JLCC_const * V * C.F_RT / (JE - 1);
    sv[SV_CAI] = g[3];
    sv[SV_CANSR] = g[4];
}

// The same with the terms evaluated here, one after the other.
GW_HD bool glob_increment(const CellStatic &C, const double *g, const Carry &cy, double Istim, double dt, double *d) {
    double T[kNT];
    glob_terms(C, g, T);
    return glob_increment(C, g, cy, Istim, dt, T, d);
}
GW_HD void step_values(const CellStatic &C, const double *g, double *sv) {
    double S[kNS];
    for (int k = 0; k < kNS; ++k) S[k] = sv_term(C, g, k);
    step_values(C, g, S, sv);
}

// dJM/dV and dJE/dV of the JLCC factors: JE = exp(2 V F/RT), JM = JLCC_const V F/RT / (JE - 1).
GW_HD void jlcc_factor_derivs(const CellStatic &C, double V, double JE, double &dJM, double &dJE) {
    dJE = 2.0 * C.F_RT * JE;
    dJM = C.JLCC_const * C.F_RT * ((JE - 1.0) - V * dJE) / sqd(JE - 1.0);
}

// The adjoint of one global increment, in kAdjParts independent parts: with lam = dL/dG[s+1] and
// G[s+1] = G[s] + d, part q adds its share of dL/dG[s] to lam_g, of dL/d(carry JLCC, Jtr, Jxfer) to
// lam_cy and of the relative sensitivities of GKr, GKs, GK1, INaKmax and Vmax to lam_th.  The sum of
// the parts is the whole adjoint (part 0 carries the identity); each part converts its own V, exp(-VF/RT)
// and Nernst-potential accumulators at its end, so that a block can run the parts one per thread.
enum AdjPart { AP_NA = 0, AP_NAK, AP_TO, AP_K1, AP_CA, AP_GATE_MH, AP_GATE_JX, AP_KR, AP_KV43, AP_KV14, kAdjParts };

GW_HD void glob_increment_adj(const CellStatic &C, const double *g, const Carry &cy, double dt, const double *T,
                              const double *lam, int part, double *lam_g, double *lam_cy, double *lam_th) {
    const gw_params &p = C.p;
    const double V = g[0], Nai = g[1], Ki = g[2], Cai = g[3], CaNSR = g[4], CaLT = g[5], CaHT = g[6];
    const double m = g[7], h = g[8], jg = g[9], xKs = g[10];
    const double *Kr = g + 11, *Kv43 = g + 16, *Kv14 = g + 26;
    const double F_RT = C.F_RT, RT_F = C.RT_F, CSA = C.CSA_FVcyto;
    const double VF_RT = V * F_RT, e = T[T_E];
    const double ENa = T[T_LNA] * RT_F, EK = T[T_LK] * RT_F, ECa = T[T_LK] * RT_F / 2.0;
    // adjoints of the currents: d[0] = dt (Istim - sum I), d[1] and d[2] their Na and K shares, d[3] the
    // buffered cytosolic Ca balance (lQ = lam3 dt beta), d[4] the NSR balance
    const double l0 = -dt * lam[0], l1 = -dt * CSA * lam[1], l2 = -dt * CSA * lam[2];
    auto beta_cyto = [&]() { return 1.0 / (1.0 + C.CMDN_const / sqd(p.KCMDN + Cai)); };
    double lV = 0, lNai = 0, lKi = 0, lCai = 0, lCaNSR = 0, lVF = 0, le = 0, lENa = 0, lEK = 0, lECa = 0;
    switch (part) {
    case AP_NA: {
        for (int i = 0; i < kNumGlobals; ++i) lam_g[i] += lam[i];
        const double lQ = lam[3] * dt * beta_cyto();
        const double lINa = l0 + l1, lINab = l0 + l1, lINaCa = l0 + 3 * l1 + CSA * lQ;
        const double m3hj = cubed(m) * h * jg;
        lam_g[7] += lINa * 3 * p.GNa * sqd(m) * h * jg * (V - ENa);
        lam_g[8] += lINa * p.GNa * cubed(m) * jg * (V - ENa);
        lam_g[9] += lINa * p.GNa * cubed(m) * h * (V - ENa);
        lV += lINa * p.GNa * m3hj + lINab * p.GNab;
        lENa -= lINa * p.GNa * m3hj + lINab * p.GNab;
        const double e1 = T[T_E1], e2 = e1 * e;
        const double numNC = e1 * cubed(Nai) * p.Cao - e2 * C.Nao3 * Cai, denNC = 1.0 + p.ksat * e2;
        const double rden = 1.0 / denNC;
        const double INaCa = C.INaCa_const * numNC * rden;
        const double lnum = lINaCa * C.INaCa_const * rden;
        const double lden = -lINaCa * INaCa * rden;
        double le1 = lnum * cubed(Nai) * p.Cao;
        lNai += lnum * 3 * e1 * sqd(Nai) * p.Cao;
        const double le2 = -lnum * C.Nao3 * Cai + lden * p.ksat;
        lCai += -lnum * e2 * C.Nao3;
        le1 += le2 * e;
        le += le2 * e1;
        lVF += le1 * p.eta * e1;
        break;
    }
    case AP_NAK: {
        const double lINaK = l0 + 3 * l1 - 2 * l2, lIKr = l0 + l2, lIKs = l0 + l2;
        const double E1k = T[T_ENAK];
        const double fNaK = 1.0 / (1.0 + 0.1245 * E1k + 0.0365 * C.sigma * e);
        const double rq = 1.0 / (1.0 + T[T_PNAK]);
        const double INaK = C.INaK_const * fNaK * rq;
        const double lf = lINaK * C.INaK_const * rq;
        const double lq = -lINaK * INaK * rq;
        lNai += lq * (-1.5 * T[T_PNAK] / Nai);
        const double lD = -lf * sqd(fNaK);
        lVF += lD * 0.1245 * (-0.1) * E1k;
        le += lD * 0.0365 * C.sigma;
        lam_th[TH_INAK] += lINaK * INaK;
        const double ERk = T[T_RKR], RKr = 1.0 / (1.0 + 1.4945 * ERk);
        const double k = p.GKr * C.sqrtKo * 0.5;
        lam_g[14] += lIKr * k * RKr * (V - EK);
        const double dRKr = -sqd(RKr) * 1.4945 * 0.0446 * ERk;
        lV += lIKr * k * Kr[3] * (RKr + (V - EK) * dRKr);
        lEK -= lIKr * k * RKr * Kr[3];
        lam_th[TH_GKR] += lIKr * (k * RKr * Kr[3] * (V - EK));
        const double sKs = Ki + 0.01833 * Nai, EKs = T[T_LKS] * RT_F;
        lam_g[10] += lIKs * 2 * p.GKs * xKs * (V - EKs);
        lV += lIKs * p.GKs * sqd(xKs);
        const double lEKs = -lIKs * p.GKs * sqd(xKs), rs = RT_F / sKs;
        lKi -= lEKs * rs;
        lNai -= lEKs * 0.01833 * rs;
        lam_th[TH_GKS] += lIKs * (p.GKs * sqd(xKs) * (V - EKs));
        break;
    }
    case AP_TO: {
        const double lIto1 = l0 + l2, lIto2 = l0;
        const double P14 = C.PKv14_Csc * kFaradayA, r1 = 1.0 / (1 - e);
        const double A14 = (Ki - p.Ko * e) + 0.02 * (Nai - p.Nao * e);
        const double mm = P14 * VF_RT * Kv14[4] * r1;
        const double lmm = lIto1 * A14 * 1.0e9, lA = lIto1 * mm * 1.0e9;
        lKi += lA;
        lNai += 0.02 * lA;
        le += lA * (-p.Ko - 0.02 * p.Nao);
        lam_g[30] += lmm * P14 * VF_RT * r1;
        lVF += lmm * P14 * Kv14[4] * r1;
        le += lmm * P14 * VF_RT * Kv14[4] * r1 * r1;
        lam_g[20] += lIto1 * p.GKv43 * (V - EK);
        lV += lIto1 * p.GKv43 * Kv43[4];
        lEK -= lIto1 * p.GKv43 * Kv43[4];
        const double r2 = 1.0 / (e - 1.0);
        const double B = (p.Clcyto * e - p.Clo) * r2, k = cy.clch * C.Ito2_const;
        lVF += lIto2 * k * B;
        le += lIto2 * k * VF_RT * (p.Clo - p.Clcyto) * r2 * r2;
        break;
    }
    case AP_K1: {
        const double lIK1 = l0 + l2, lIKp = l0 + l2;
        const double lQ = lam[3] * dt * beta_cyto();
        const double lICab = l0 - 0.5 * CSA * lQ, lIpCa = l0 - 0.5 * CSA * lQ;
        const double uK1 = V - EK, EK1 = T[T_K1], K1inf = 1.0 / (2.0 + EK1);
        const double dK1 = -sqd(K1inf) * 1.5 * F_RT * EK1;
        const double dIdu = p.GK1 * C.IK1_const * (K1inf + uK1 * dK1);
        lV += lIK1 * dIdu;
        lEK -= lIK1 * dIdu;
        lam_th[TH_GK1] += lIK1 * (p.GK1 * K1inf * C.IK1_const * uK1);
        const double EKp = T[T_KP], Kp = 1. / (1. + EKp);
        const double dKp = sqd(Kp) * EKp / 5.98;
        lV += lIKp * p.GKp * (Kp + (V - EK) * dKp);
        lEK -= lIKp * p.GKp * Kp;
        lam_cy[0] += l0 * C.ICaL_const;  // ICaL = sum JLCC x ICaL_const
        lV += lICab * p.GCab;
        lECa -= lICab * p.GCab;
        lCai += lIpCa * p.IpCamax * p.KmpCa / sqd(p.KmpCa + Cai);
        break;
    }
    case AP_CA: {
        const double beta = beta_cyto(), lQ = lam[3] * dt * beta;
        const double fu = T[T_FU], ru = T[T_RU], rd = 1.0 / (1.0 + fu + ru);
        const double Jup = (p.Vmaxf * fu - p.Vmaxr * ru) * rd;
        const double dLT = p.kLTRPNp * Cai * (p.LTRPNtot - CaLT) - p.kLTRPNm * CaLT;
        const double dHT = p.kHTRPNp * Cai * (p.HTRPNtot - CaHT) - p.kHTRPNm * CaHT;
        const double e1 = T[T_E1], e2 = e1 * e;
        const double INaCa = C.INaCa_const * (e1 * cubed(Nai) * p.Cao - e2 * C.Nao3 * Cai) / (1.0 + p.ksat * e2);
        const double ICab = p.GCab * (V - ECa), IpCa = p.IpCamax * (Cai / (p.KmpCa + Cai));
        const double Q3 =
            -0.5 * CSA * (ICab + IpCa - 2 * INaCa) + C.VSS_Vcyto * (cy.jxfer * C.CRU_factor) - Jup - (dLT + dHT);
        const double lbeta = lam[3] * dt * Q3;
        const double lJup = -lQ + dt * C.Vcyto_VNSR * lam[4];
        const double ldLT = -lQ + dt * lam[5], ldHT = -lQ + dt * lam[6];
        const double dJdf = (p.Vmaxf * (1.0 + ru) + p.Vmaxr * ru) * rd * rd;
        const double dJdr = -(p.Vmaxr * (1.0 + fu) + p.Vmaxf * fu) * rd * rd;
        lCai += lJup * dJdf * p.Hf * fu / Cai;
        lCaNSR += lJup * dJdr * p.Hr * ru / CaNSR;
        lam_th[TH_VMAX] += lJup * Jup;
        lam_cy[1] += -dt * C.VJSR_VNSR * lam[4] * C.CRU_factor;
        lam_cy[2] += C.VSS_Vcyto * lQ * C.CRU_factor;
        lCai += lbeta * sqd(beta) * 2.0 * C.CMDN_const / cubed(p.KCMDN + Cai);
        lCai += ldLT * p.kLTRPNp * (p.LTRPNtot - CaLT) + ldHT * p.kHTRPNp * (p.HTRPNtot - CaHT);
        lam_g[5] += ldLT * (-p.kLTRPNp * Cai - p.kLTRPNm);
        lam_g[6] += ldHT * (-p.kHTRPNp * Cai - p.kHTRPNm);
        break;
    }
    case AP_GATE_MH:
    case AP_GATE_JX: {
        const Gates gr = gate_rates(V, true, T);
        if (part == AP_GATE_MH) {
            lam_g[7] += lam[7] * dt * (-gr.am - gr.bm);
            lam_g[8] += lam[8] * dt * (-gr.ah - gr.bh);
            lV += lam[7] * dt * (gr.dam * (1.0 - m) - gr.dbm * m);
            lV += lam[8] * dt * (gr.dah * (1.0 - h) - gr.dbh * h);
        } else {
            lam_g[9] += lam[9] * dt * (-gr.aj - gr.bj);
            lam_g[10] += -lam[10] * dt * gr.tinv;
            lV += lam[9] * dt * (gr.daj * (1.0 - jg) - gr.dbj * jg);
            lV += lam[10] * dt * (gr.dxinf * gr.tinv + (gr.xinf - xKs) * gr.dtinv);
        }
        break;
    }
    case AP_KR: {
        // IKr chain: d_k = dt (sum over edges a->b of q x_a into b, minus out of a)
        const KrQ q = kr_q(T);
        const double *l = lam + 11;
        double *lx = lam_g + 11;
        double lq01 = 0, lq10 = 0, lq23 = 0, lq24 = 0, lq32 = 0, lq34 = 0, lq43 = 0, lq42 = 0;
        auto edge = [&](int a, int b, double qv, double *lqv) {
            const double w = dt * (l[b] - l[a]);
            lx[a] += qv * w;
            if (lqv) *lqv += Kr[a] * w;
        };
        edge(0, 1, q.q01, &lq01);
        edge(1, 0, q.q10, &lq10);
        edge(1, 2, p.Kf, nullptr);
        edge(2, 1, p.Kb, nullptr);
        edge(2, 3, q.q23, &lq23);
        edge(2, 4, q.q24, &lq24);
        edge(3, 2, q.q32, &lq32);
        edge(3, 4, q.q34, &lq34);
        edge(4, 3, q.q43, &lq43);
        edge(4, 2, q.q42, &lq42);
        // q42 = q32 q43 q24 / (q23 q34)
        lq32 += lq42 * q.q42 / q.q32;
        lq43 += lq42 * q.q42 / q.q43;
        lq24 += lq42 * q.q42 / q.q24;
        lq23 -= lq42 * q.q42 / q.q23;
        lq34 -= lq42 * q.q42 / q.q34;
        lV += lq01 * 0.0272 * q.q01 + lq10 * (-0.0431) * q.q10 + lq23 * 0.0262 * q.q23 + lq24 * 2.71e-6 * q.q24 +
              lq32 * (-0.0269) * q.q32 + lq34 * 0.0120 * q.q34 + lq43 * (-0.0443) * q.q43;
        break;
    }
    default: {  // AP_KV43, AP_KV14
        const int ch = part == AP_KV14 ? 0 : 1;
        const double *x = ch == 0 ? Kv14 : Kv43;
        const double *l = lam + (ch == 0 ? 26 : 16);
        double *lx = lam_g + (ch == 0 ? 26 : 16);
        double r[4], lr[4] = {0, 0, 0, 0};
        kv_rates(p, ch, T, r);
        KvEdge E[26];
        kv_edges(p, ch, E);
        for (int k = 0; k < 26; ++k) {
            const double qv = E[k].coef * r[E[k].rate];
            const double w = dt * (l[E[k].b] - l[E[k].a]);
            lx[E[k].a] += qv * w;
            lr[E[k].rate] += E[k].coef * x[E[k].a] * w;
        }
        const double ka = ch == 0 ? p.aaKv14 : p.aaKv43, ki = ch == 0 ? p.aiKv14 : p.aiKv43;
        const double kb = ch == 0 ? p.baKv14 : p.baKv43, kbi = ch == 0 ? p.biKv14 : p.biKv43;
        lV += lr[0] * ka * r[0] - lr[1] * ki * r[1] - lr[2] * kb * r[2] + lr[3] * kbi * r[3];
        break;
    }
    }
    // this part's Nernst potentials, VF_RT and e = exp(-VF_RT) back to the globals
    if (lENa != 0.0) lNai += lENa * (-RT_F / Nai);
    if (lEK != 0.0 || lECa != 0.0) lKi += lEK * (-RT_F / Ki) + lECa * (-RT_F / (2.0 * Ki));
    lV += F_RT * lVF - F_RT * e * le;
    lam_g[0] += lV;
    lam_g[1] += lNai;
    lam_g[2] += lKi;
    lam_g[3] += lCai;
    lam_g[4] += lCaNSR;
}

// All parts, one after the other.
GW_HD void glob_increment_adj(const CellStatic &C, const double *g, const Carry &cy, double dt, const double *T,
                              const double *lam, double *lam_g, double *lam_cy, double *lam_th) {
    for (int q = 0; q < kAdjParts; ++q) glob_increment_adj(C, g, cy, dt, T, lam, q, lam_g, lam_cy, lam_th);
}

// ---------------------------------------------------------------------------------------------
// One CRU over one global step, given its jump trajectory: sub-steps of lengths h_k separated by
// events.  The arithmetic of the sub-step and of the events is the FP64 SSA lane's
// (SsaLane<double, true> in gw_kernel.cuh, the reference's order), so that a replay of the
// trajectory at the recording's parameters gives the recording's values bit for bit.
// ---------------------------------------------------------------------------------------------

// Continuous state of a CRU within a step.
struct CruCont {
    double c[4], J, L[4], rel[4];
};

// Per-step inputs of a CRU from its cell, and the parameters it uses.
struct CruIn {
    double Cai, CaNSR, JM, JE;
};
struct CruPar {
    double rRyR, rtr, riss, rxfer, KBSR, KBSL, BSR_const, BSL_const, KCSQN, CSQN_const, VSS_VJSR, Cao_scaled;
};
GW_HD CruPar cru_par(const CellStatic &C) {
    return CruPar{C.p.rRyR, C.p.rtr, C.p.riss, C.p.rxfer, C.p.KBSR, C.p.KBSL, C.BSR_const, C.BSL_const,
                  C.p.KCSQN, C.CSQN_const, C.VSS_VJSR, C.Cao_scaled};
}

// Event effects on the continuous state (sample_new_state, SSA.tpp:262-283): a subunit starting
// to conduct (LCC open, voltage gate not inactivated) sets JLCC from CaSS; one that stops sets
// it to 0; a RyR transition resets Jrel with the new open count; other events change nothing
// continuous but end a sub-step.
enum CruEvent { EV_NONE = 0, EV_JLCC_SET = 1, EV_JLCC_ZERO = 2, EV_JREL = 3 };

// Jrel at the start of the step from the open counts o (copy_from_CRUState, SSA.tpp:10-33).
GW_HD void cru_begin(CruCont &s, const int o[4], const CruPar &P) {
    for (int j = 0; j < 4; ++j) s.rel[j] = P.rRyR * (double)o[j] * (s.J - s.c[j]);
}

// One sub-step of length h (update_fluxes, update_CaSS, update_CaJSR); returns the fluxes taken at
// its start (the step's carry when it is the last one).
GW_HD void cru_substep(CruCont &s, double h, const CruIn &in, const CruPar &P, double &jtr, double &jxfer_sum) {
    double jiss[4], jxf[4];
    jtr = P.rtr * (in.CaNSR - s.J);
    jiss[0] = P.riss * (s.c[1] + s.c[3] - 2.0 * s.c[0]);
    jiss[1] = P.riss * (s.c[2] + s.c[0] - 2.0 * s.c[1]);
    jiss[2] = P.riss * (s.c[3] + s.c[1] - 2.0 * s.c[2]);
    jiss[3] = P.riss * (s.c[0] + s.c[2] - 2.0 * s.c[3]);
    for (int j = 0; j < 4; ++j) jxf[j] = P.rxfer * (s.c[j] - in.Cai);
    double cn[4];
    for (int j = 0; j < 4; ++j) {
        const double x = s.c[j];
        const double beta = 1.0 / (1.0 + (P.BSR_const / ((P.KBSR + x) * (P.KBSR + x))) +
                                   (P.BSL_const / ((P.KBSL + x) * (P.KBSL + x))));
        cn[j] = x + h * (s.L[j] + s.rel[j] - jxf[j] + jiss[j]) * beta;
    }
    {
        const double x = s.J;
        const double beta = 1.0 / (1.0 + P.CSQN_const / ((P.KCSQN + x) * (P.KCSQN + x)));
        s.J += h * beta * (jtr - P.VSS_VJSR * (s.rel[0] + s.rel[1] + s.rel[2] + s.rel[3]));
    }
    for (int j = 0; j < 4; ++j) s.c[j] = cn[j];
    jxfer_sum = jxf[0] + jxf[1] + jxf[2] + jxf[3];
}

GW_HD void cru_event(CruCont &s, int ev, int j, int onew, const CruIn &in, const CruPar &P) {
    if (ev == EV_JLCC_SET)
        s.L[j] = in.JM * (P.Cao_scaled - in.JE * s.c[j]);
    else if (ev == EV_JLCC_ZERO)
        s.L[j] = 0.0;
    else if (ev == EV_JREL)
        s.rel[j] = P.rRyR * (double)onew * (s.J - s.c[j]);
}

// Adjoint accumulators of a CRU's per-step inputs and parameters.
struct CruAdjIn {
    double Cai, CaNSR, JM, JE, rRyR_rel, CSQN;  // rRyR_rel: rRyR dL/drRyR; CSQN: dL/dCSQN_const
};

// Adjoint of cru_event; s is the state the event acts on (after the sub-step; an event changes
// neither CaSS nor CaJSR).  la: adjoints of the state after the event; on return, before it.
GW_HD void cru_event_adj(const CruCont &s, int ev, int j, int onew, const CruIn &in, const CruPar &P, CruCont &la,
                         CruAdjIn &ai) {
    if (ev == EV_JLCC_SET) {
        const double l = la.L[j];
        ai.JM += l * (P.Cao_scaled - in.JE * s.c[j]);
        ai.JE += l * (-in.JM * s.c[j]);
        la.c[j] += l * (-in.JM * in.JE);
        la.L[j] = 0.0;
    } else if (ev == EV_JLCC_ZERO) {
        la.L[j] = 0.0;
    } else if (ev == EV_JREL) {
        const double l = la.rel[j], k = P.rRyR * (double)onew;
        ai.rRyR_rel += l * k * (s.J - s.c[j]);
        la.J += l * k;
        la.c[j] -= l * k;
        la.rel[j] = 0.0;
    }
}

// Adjoint of cru_substep from its start state s0 (the state before the sub-step).  la holds the
// adjoints after the sub-step (c, J, L, rel); l_jtr / l_jxfer are the adjoints of the returned
// fluxes (non-zero for the step's last sub-step, whose fluxes are the carry).
GW_HD void cru_substep_adj(const CruCont &s0, double h, const CruIn &in, const CruPar &P, double l_jtr,
                           double l_jxfer, CruCont &la, CruAdjIn &ai) {
    double jiss[4], jxf[4];
    const double jtr = P.rtr * (in.CaNSR - s0.J);
    jiss[0] = P.riss * (s0.c[1] + s0.c[3] - 2.0 * s0.c[0]);
    jiss[1] = P.riss * (s0.c[2] + s0.c[0] - 2.0 * s0.c[1]);
    jiss[2] = P.riss * (s0.c[3] + s0.c[1] - 2.0 * s0.c[2]);
    jiss[3] = P.riss * (s0.c[0] + s0.c[2] - 2.0 * s0.c[3]);
    for (int j = 0; j < 4; ++j) jxf[j] = P.rxfer * (s0.c[j] - in.Cai);
    double lc[4], liss[4], lxf[4];
    for (int j = 0; j < 4; ++j) {
        // beta = 1 / (1 + BSR/uR^2 + BSL/uL^2) and its x derivative 2 beta^2 (BSR/uR^3 + BSL/uL^3),
        // over the common denominator (one division; the adjoint need not round as the forward)
        const double x = s0.c[j];
        const double uR = P.KBSR + x, uL = P.KBSL + x, A2 = uR * uR, B2 = uL * uL;
        const double r = 1.0 / (A2 * B2 + P.BSR_const * B2 + P.BSL_const * A2);
        const double beta = A2 * B2 * r;
        const double dbeta = 2.0 * uR * uL * (P.BSR_const * uL * B2 + P.BSL_const * uR * A2) * r * r;
        const double A = s0.L[j] + s0.rel[j] - jxf[j] + jiss[j];
        const double lcn = la.c[j];
        const double lA = lcn * h * beta;
        lc[j] = lcn + lcn * h * A * dbeta;
        la.L[j] += lA;
        la.rel[j] += lA;
        lxf[j] = -lA + l_jxfer;
        liss[j] = lA;
    }
    double lJ, ljtr = l_jtr;
    {
        // beta = u^2 / (u^2 + CSQN), d beta/dx = 2 u CSQN / (u^2 + CSQN)^2,
        // d beta/dCSQN = -u^2 / (u^2 + CSQN)^2
        const double x = s0.J, u = P.KCSQN + x, U2 = u * u;
        const double r = 1.0 / (U2 + P.CSQN_const);
        const double beta = U2 * r;
        const double G = jtr - P.VSS_VJSR * (s0.rel[0] + s0.rel[1] + s0.rel[2] + s0.rel[3]);
        const double lJn = la.J;
        lJ = lJn + lJn * h * G * (2.0 * u * P.CSQN_const * r * r);
        ljtr += lJn * h * beta;
        for (int j = 0; j < 4; ++j) la.rel[j] -= lJn * h * beta * P.VSS_VJSR;
        ai.CSQN += lJn * h * G * (-U2 * r * r);
    }
    for (int j = 0; j < 4; ++j) {
        lc[j] += P.rxfer * lxf[j];
        ai.Cai -= P.rxfer * lxf[j];
    }
    lc[1] += P.riss * liss[0]; lc[3] += P.riss * liss[0]; lc[0] -= 2.0 * P.riss * liss[0];
    lc[2] += P.riss * liss[1]; lc[0] += P.riss * liss[1]; lc[1] -= 2.0 * P.riss * liss[1];
    lc[3] += P.riss * liss[2]; lc[1] += P.riss * liss[2]; lc[2] -= 2.0 * P.riss * liss[2];
    lc[0] += P.riss * liss[3]; lc[2] += P.riss * liss[3]; lc[3] -= 2.0 * P.riss * liss[3];
    ai.CaNSR += P.rtr * ljtr;
    lJ -= P.rtr * ljtr;
    for (int j = 0; j < 4; ++j) la.c[j] = lc[j];
    la.J = lJ;
}

// Adjoint of cru_begin: the step's Jrel from its start state.
GW_HD void cru_begin_adj(const CruCont &s0, const int o[4], const CruPar &P, CruCont &la, CruAdjIn &ai) {
    for (int j = 0; j < 4; ++j) {
        const double l = la.rel[j], k = P.rRyR * (double)o[j];
        ai.rRyR_rel += l * k * (s0.J - s0.c[j]);
        la.J += l * k;
        la.c[j] -= l * k;
        la.rel[j] = 0.0;
    }
}

// glob_increment_adj with the terms evaluated here.
GW_HD void glob_increment_adj(const CellStatic &C, const double *g, const Carry &cy, double dt, const double *lam,
                              double *lam_g, double *lam_cy, double *lam_th) {
    double T[kNT];
    glob_terms(C, g, T);
    glob_increment_adj(C, g, cy, dt, T, lam, lam_g, lam_cy, lam_th);
}

}  // namespace adj
}  // namespace gw
