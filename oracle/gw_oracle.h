/*
 * gw_oracle.h -- CPU oracle for the Greenstein-Winslow per-CRU hybrid SSA and FP64 global step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference's hot path
 * (lukeoloughlin/GW-model, src/includes/{GW.tpp,SSA.tpp,GW_utils.hpp,GW_utils.tpp,common.hpp}).
 * It exists to check the CUDA engine: only tests/, __graft_entry__.smoke() and the CPU-baseline
 * leg of bench.py may load it.  The product never links or calls it.
 *
 * Parity pinning: the restatement is pinned bit-for-bit against the reference's own C++ headers,
 * compiled unmodified (oracle/ref_harness.cpp + oracle/eigen_shim) with the same injected draws;
 * the golden vectors that pin it are committed under tests/golden/.
 *
 * Random draws.  The reference draws from a thread_local engine seeded by std::random_device
 * (common.hpp:19-29), which cannot be reproduced.  Every draw here (and in the CUDA engine, and in
 * the reference harness) instead comes from a counter-based stream:
 *   Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), key = {seed_lo, seed_hi},
 *   counter = {k >> 1, cru, (uint32)step, (stream << 28) | cell},
 *   64-bit word = lanes {2h+1 : 2h} with h = k & 1,
 *   U53 mode: u = max(word >> 11, 1) * 2^-53     (FP64 engine)
 *   U24 mode: u = max(word >> 40, 1) * 2^-24     (FP32 engine; exactly representable in float)
 * where k counts the draws a CRU makes inside one global step, in the reference's call order.
 */
#ifndef GW_ORACLE_H
#define GW_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* X-macro over the reference's Parameters struct (GW_utils.hpp:40-156): (type, name, default). */
#define ORC_PARAM_FIELDS(X) \
    X(double, T, 310.0) X(double, CSA, 153.4) X(double, Vcyto, 25.84) X(double, VNSR, 1.113) \
    X(double, VJSR, 22.26e-6) X(double, VSS, 0.2303e-6) X(int, NCaRU, 12500) X(double, Ko, 4.0) \
    X(double, Nao, 138.0) X(double, Cao, 2.0) X(double, Clo, 150.0) X(double, Clcyto, 20.0) \
    X(double, f, 0.85) X(double, g, 2.0) X(double, f1, 0.005) X(double, g1, 7.0) X(double, a, 2.0) \
    X(double, b, 1.9356) X(double, gamma0, 0.44) X(double, omega, 0.02158) X(double, PCaL, 9.13e-13) \
    X(double, kfClCh, 13.3156) X(double, kbClCh, 2.0) X(double, Pto2, 2.65e-15) \
    X(double, k12, 877.5) X(double, k21, 250.0) X(double, k23, 2.358e8) X(double, k32, 9.6) \
    X(double, k34, 1.415e6) X(double, k43, 13.65) X(double, k45, 0.07) X(double, k54, 93.385) \
    X(double, k56, 1.887e7) X(double, k65, 30.0) X(double, k25, 2.358e6) X(double, k52, 0.001235) \
    X(double, rRyR, 3.92) X(double, rxfer, 200.0) X(double, rtr, 0.333) X(double, riss, 20.0) \
    X(double, BSRT, 0.047) X(double, KBSR, 0.00087) X(double, BSLT, 1.124) X(double, KBSL, 0.0087) \
    X(double, CSQNT, 13.5) X(double, KCSQN, 0.63) X(double, CMDNT, 0.05) X(double, KCMDN, 0.00238) \
    X(double, GNa, 12.8) X(double, GKr, 0.024) X(double, Kf, 0.0266) X(double, Kb, 0.1348) \
    X(double, GKs, 0.00271) X(double, GKv43, 0.1389) X(double, alphaa0Kv43, 0.5437) \
    X(double, aaKv43, 0.02898) X(double, betaa0Kv43, 0.08019) X(double, baKv43, 0.04684) \
    X(double, alphai0Kv43, 0.04984) X(double, aiKv43, 3.37302e-4) X(double, betai0Kv43, 8.1948e-4) \
    X(double, biKv43, 5.374e-8) X(double, f1Kv43, 1.8936) X(double, f2Kv43, 14.225) \
    X(double, f3Kv43, 158.574) X(double, f4Kv43, 142.937) X(double, b1Kv43, 6.7735) \
    X(double, b2Kv43, 15.621) X(double, b3Kv43, 28.753) X(double, b4Kv43, 524.576) \
    X(double, PKv14, 1.989e-7) X(double, alphaa0Kv14, 1.8931) X(double, aaKv14, 0.006950) \
    X(double, betaa0Kv14, 0.01179) X(double, baKv14, 0.08527) X(double, alphai0Kv14, 0.002963) \
    X(double, aiKv14, 0.0) X(double, betai0Kv14, 1.0571e-4) X(double, biKv14, 0.0) \
    X(double, f1Kv14, 0.2001) X(double, f2Kv14, 0.3203) X(double, f3Kv14, 13.509) \
    X(double, f4Kv14, 1151.765) X(double, b1Kv14, 2.230) X(double, b2Kv14, 12.0) \
    X(double, b3Kv14, 5.370) X(double, b4Kv14, 5.240) X(double, Csc, 1.0e6) X(double, GK1, 3.0) \
    X(double, KmK1, 13.0) X(double, GKp, 0.002659) X(double, kNaCa, 0.27) X(double, KmNa, 87.5) \
    X(double, KmCa, 1.38) X(double, ksat, 0.2) X(double, eta, 0.35) X(double, INaKmax, 0.901) \
    X(double, KmNai, 10.0) X(double, KmKo, 1.5) X(double, IpCamax, 0.03) X(double, KmpCa, 0.0005) \
    X(double, GCab, 0.0002536) X(double, GNab, 0.00264) X(double, kHTRPNp, 20.0) \
    X(double, kHTRPNm, 6.60e-5) X(double, kLTRPNp, 40.0) X(double, kLTRPNm, 0.04) \
    X(double, HTRPNtot, 0.140) X(double, LTRPNtot, 0.070) X(double, Vmaxf, 0.0002096) \
    X(double, Vmaxr, 0.0002096) X(double, Kmf, 0.000260) X(double, Kmr, 1.8) X(double, Hf, 0.75) \
    X(double, Hr, 0.75)

#define ORC_DECL_FIELD(t, n, d) t n;
typedef struct orc_params { ORC_PARAM_FIELDS(ORC_DECL_FIELD) } orc_params;
#undef ORC_DECL_FIELD

/* GW::GlobalState (GW_utils.hpp:229-252), same member order. */
typedef struct orc_globals {
    double V, Nai, Ki, Cai, CaNSR, CaLTRPN, CaHTRPN, m, h, j, xKs;
    double Kr[5];
    double Kv43[10];
    double Kv14[10];
} orc_globals;

/* Flat record of the reference's Constants (GW_utils.hpp:162-227), same member order. */
typedef struct orc_consts {
    double RT_F, F_RT, CRU_factor, CSA_FVcyto, VSS_Vcyto, Vcyto_VNSR, VJSR_VNSR;
    double a, gamma0, gamma0a, gamma0a2, gamma0a3, gamma0a4, binv, omega, omega_b, omega_b2,
        omega_b3, omega_b4;
    double BSR_const, BSL_const, VSS_VJSR, CSQN_const, JLCC_const, Cao_scaled, Nao3, INaCa_const,
        sigma, INaK_const, sqrtKo, PKv14_Csc, Ito2_const, IK1_const, ICaL_const, CMDN_const;
    double VF_RT, expmVF_RT, ENa, EK, ECa, beta_cyto, JLCC_multiplier, JLCC_exp, alphaLCC, betaLCC,
        yinfLCC, tauLCC;
} orc_consts;

/* GW::Currents (GW.hpp:24-42). */
typedef struct orc_currents {
    double INa, INab, INaCa, INaK, IKr, IKs, Ito1, Ito2, IK1, IKp, ICaL, ICab, IpCa, Jup, Jtr_tot,
        Jxfer_tot;
} orc_currents;

enum { ORC_U53 = 0, ORC_U24 = 1 };
enum { ORC_STREAM_SSA = 0, ORC_STREAM_INIT = 1 };

typedef struct orc_model orc_model;

/* ---- parameters / constants / RNG ---- */
void orc_params_default(orc_params *p);
int orc_param_count(void);
void orc_globals_default(orc_globals *g);     /* GW::GlobalState defaults (GW_utils.hpp:231-247) */
void orc_globals_py_default(orc_globals *g);  /* GWGlobalState() defaults (pyGW.cpp:31-76) */
void orc_constants(const orc_params *p, int nCRU, orc_consts *c);
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
/* n uniforms of the stream (seed, cell, cru, step, stream), draws k0 .. k0+n-1. */
void orc_uniforms(uint64_t seed, uint32_t cell, uint32_t cru, uint64_t step, uint32_t stream,
                  int umode, uint32_t k0, int n, double *out);

/* ---- per-CRU kernels (known-answer tests) ---- */
/* LCC (3 per subunit), inactivation, RyR (12 per subunit), ClCh rates and subunit totals
 * for one CRU given its channel states and CaSS (update_rates, SSA.tpp:48-56). */
void orc_cru_rates(const orc_params *p, const orc_consts *c, const int *LCC, const int *LCCi,
                   const int *RyR, const int *ClCh, const double *CaSS, double *LCC_rates,
                   double *LCCi_rates, double *RyR_rates, double *ClCh_rates,
                   double *subunit_rates);
/* Per-step voltage constants set by GW_model::SSA (GW.tpp:216-221) into c. */
void orc_ssa_step_constants(orc_consts *c, double V);

/* ---- model ---- */
orc_model *orc_create(const orc_params *p, int nCRU, uint64_t seed, uint32_t cell, int umode);
void orc_destroy(orc_model *m);
int orc_ncru(const orc_model *m);
void orc_set_globals(orc_model *m, const orc_globals *g);
void orc_get_globals(const orc_model *m, orc_globals *g);
/* CRU arrays in the reference's layouts: CaSS [n,4], CaJSR [n], LCC/LCCi/ClCh [n,4],
 * RyR [n,4,6].  Any pointer may be NULL on get. */
void orc_set_crus(orc_model *m, const double *CaSS, const double *CaJSR, const int *LCC,
                  const int *LCCi, const int *RyR, const int *ClCh);
void orc_get_crus(const orc_model *m, double *CaSS, double *CaJSR, int *LCC, int *LCCi, int *RyR,
                  int *ClCh);
/* Per-CRU flux carry: JLCC [n,4] (stateful), Jxfer [n,4], Jtr [n] (last update_fluxes). */
void orc_set_fluxes(orc_model *m, const double *JLCC, const double *Jxfer, const double *Jtr);
void orc_get_fluxes(const orc_model *m, double *JLCC, double *Jxfer, double *Jtr);
void orc_get_consts(const orc_model *m, orc_consts *c);
void orc_get_currents(const orc_model *m, orc_currents *cur);
void orc_set_step(orc_model *m, uint64_t step);
uint64_t orc_get_step(const orc_model *m);
/* Draws the reference's random initial CRU state (GW_utils.tpp:5-64) from stream INIT. */
void orc_sample_initial_crus(orc_model *m);
/* One global step (GW_model::euler_step, GW.tpp:237-272) with stimulus Istim. */
void orc_euler_step(orc_model *m, double dt, double Istim);
/* num_steps steps; Istim[i] is the stimulus of step i.  Records globals after every step i with
 * i % record_every == 0 into rec_globals[r] (r < max_records) and rec_t[r] (time after the step),
 * as pyGW.hpp:113-121 does.  Returns the number of records written. */
int64_t orc_run(orc_model *m, double dt, int64_t num_steps, const double *Istim, int record_every,
                int64_t max_records, double *rec_t, orc_globals *rec_globals);
/* orc_run recording the CRU arrays too (record_state, pyGW.hpp:56-99): record r of CaSS is
 * rec_CaSS[r][n][4], of RyR rec_RyR[r][n][4][6], and so on; NULL skips a field.  Returns the
 * number of records the reference's loop makes, ceil(num_steps / record_every); the first
 * max_records are stored. */
int64_t orc_run_record(orc_model *m, double dt, int64_t num_steps, const double *Istim,
                       int record_every, int64_t max_records, double *rec_t,
                       orc_globals *rec_globals, double *rec_CaSS, double *rec_CaJSR,
                       int *rec_LCC, int *rec_LCCi, int *rec_RyR, int *rec_ClCh);
/* Total SSA events (jumps) executed so far, and the worst per-CRU-step count. */
int64_t orc_event_count(const orc_model *m);
int orc_set_threads(int n);

#ifdef __cplusplus
}
#endif
#endif
