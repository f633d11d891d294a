/*
 * gw_oracle.c -- CPU oracle (TEST INFRASTRUCTURE ONLY; see gw_oracle.h).
 *
 * Plain-C restatement of the reference's per-CRU hybrid SSA and FP64 global step.  Every function
 * cites the reference file:line it follows and keeps the reference's expression order, so that
 * with -ffp-contract=off it reproduces the reference's arithmetic exactly under the same draws.
 * The product never links this file.
 */
#include "gw_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define FARADAY 96.5   /* common.hpp:9 */
#define GAS_CONST 8.314 /* common.hpp:10 */

static inline double sq(double x) { return x * x; }     /* common.hpp:12-13 */
static inline double cube(double x) { return x * x * x; } /* common.hpp:15-16 */

/* ------------------------------------------------------------------------------------------ */
/* parameters and constants                                                                    */
/* ------------------------------------------------------------------------------------------ */

void orc_params_default(orc_params *p) {
#define SET_DEFAULT(t, n, d) p->n = (t)(d);
    ORC_PARAM_FIELDS(SET_DEFAULT)
#undef SET_DEFAULT
}

int orc_param_count(void) {
    int n = 0;
#define COUNT(t, nm, d) ++n;
    ORC_PARAM_FIELDS(COUNT)
#undef COUNT
    return n;
}

/* GW_utils.hpp:231-247 */
void orc_globals_default(orc_globals *g) {
    static const double Kr[5] = {0.999503, 4.13720e-4, 7.27568e-5, 8.73984e-6, 1.36159e-6};
    static const double Kv43[10] = {0.953060,   0.0253906,  2.53848e-4, 1.12796e-6, 1.87950e-9,
                                    0.0151370,  0.00517622, 8.96600e-4, 8.17569e-5, 2.24032e-6};
    static const double Kv14[10] = {0.722328,   0.101971,   0.00539932, 1.27081e-4, 1.82742e-6,
                                    0.152769,   0.00962328, 0.00439043, 0.00195348, 0.00143629};
    g->V = -91.382;
    g->Nai = 10.0;
    g->Ki = 131.84;
    g->Cai = 1.45273e-4;
    g->CaNSR = 0.908882;
    g->CaLTRPN = 8.98282e-3;
    g->CaHTRPN = 0.137617;
    g->m = 5.33837e-4;
    g->h = 0.996345;
    g->j = 0.997315;
    g->xKs = 2.04171e-4;
    memcpy(g->Kr, Kr, sizeof Kr);
    memcpy(g->Kv43, Kv43, sizeof Kv43);
    memcpy(g->Kv14, Kv14, sizeof Kv14);
}

/* pyGW.cpp:31-76: identical except CaLTRPN = 8.9282e-3. */
void orc_globals_py_default(orc_globals *g) {
    orc_globals_default(g);
    g->CaLTRPN = 8.9282e-3;
}

/* Constants ctor, GW_utils.tpp:67-116. */
void orc_constants(const orc_params *p, int nCRU, orc_consts *c) {
    memset(c, 0, sizeof *c);
    c->RT_F = GAS_CONST * p->T / FARADAY;
    c->F_RT = 1.0 / c->RT_F;
    c->CRU_factor = (double)p->NCaRU / (double)nCRU;
    c->CSA_FVcyto = p->CSA / (1000 * p->Vcyto * FARADAY);
    c->VSS_Vcyto = p->VSS / p->Vcyto;
    c->Vcyto_VNSR = p->Vcyto / p->VNSR;
    c->VJSR_VNSR = p->VJSR / p->VNSR;
    c->a = p->a;
    c->gamma0 = p->gamma0;
    c->gamma0a = c->gamma0 * p->a;
    c->gamma0a2 = c->gamma0a * p->a;
    c->gamma0a3 = c->gamma0a2 * p->a;
    c->gamma0a4 = c->gamma0a3 * p->a;
    c->binv = 1.0 / p->b;
    c->omega = p->omega;
    c->omega_b = c->omega * c->binv;
    c->omega_b2 = c->omega_b * c->binv;
    c->omega_b3 = c->omega_b2 * c->binv;
    c->omega_b4 = c->omega_b3 * c->binv;
    c->BSR_const = p->KBSR * p->BSRT;
    c->BSL_const = p->KBSL * p->BSLT;
    c->VSS_VJSR = p->VSS / p->VJSR;
    c->CSQN_const = p->KCSQN * p->CSQNT;
    c->JLCC_const = 2.0e6 * p->PCaL / p->VSS;
    c->Cao_scaled = 0.341 * p->Cao;
    c->Nao3 = p->Nao * p->Nao * p->Nao;
    c->INaCa_const = 5000.0 * p->kNaCa /
                     ((p->KmNa * p->KmNa * p->KmNa + p->Nao * p->Nao * p->Nao) * (p->KmCa + p->Cao));
    c->sigma = (exp(p->Nao / 67.3) - 1.0) / 7.0;
    c->INaK_const = p->INaKmax * p->Ko / (p->Ko + p->KmKo);
    c->sqrtKo = sqrt(p->Ko);
    c->PKv14_Csc = p->PKv14 / p->Csc;
    c->Ito2_const = 1.0e9 * p->Pto2 * FARADAY * c->CRU_factor / p->CSA;
    c->IK1_const = p->Ko / (p->Ko + p->KmK1);
    c->ICaL_const = -1000.0 * (2.0 * FARADAY * p->VSS) * c->CRU_factor / p->CSA;
    c->CMDN_const = p->KCMDN * p->CMDNT;
}

/* GW_model::SSA, GW.tpp:216-221 (alphaLCC..tauLCC: GW_utils.hpp:365-375). */
void orc_ssa_step_constants(orc_consts *c, double V) {
    c->alphaLCC = 2.0 * exp(0.012 * (V - 35.0));
    c->betaLCC = 0.0882 * exp(-0.05 * (V - 35.0));
    c->yinfLCC = 0.4 / (1.0 + exp((V + 12.5) / 5.0)) + 0.6;
    c->tauLCC = 340.0 / (1.0 + exp((V + 30.0) / 12.0)) + 60.0;
    c->JLCC_exp = sq(1.0 / c->expmVF_RT);
    c->JLCC_multiplier = c->JLCC_const * V * c->F_RT / (c->JLCC_exp - 1);
}

/* ------------------------------------------------------------------------------------------ */
/* counter-based draws (replace common.hpp:19-29)                                              */
/* ------------------------------------------------------------------------------------------ */

void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        c1 = (uint32_t)p1;
        c3 = (uint32_t)p0;
        c0 = n0;
        c2 = n2;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

typedef struct orc_stream {
    uint32_t key[2];
    uint32_t ctr[4];
    uint32_t buf[4];
    uint32_t k;
    int umode;
} orc_stream;

static void stream_open(orc_stream *s, uint64_t seed, uint32_t cell, uint32_t cru, uint64_t step,
                        uint32_t stream, int umode) {
    s->key[0] = (uint32_t)seed;
    s->key[1] = (uint32_t)(seed >> 32);
    s->ctr[0] = 0;
    s->ctr[1] = cru;
    s->ctr[2] = (uint32_t)step;
    s->ctr[3] = (stream << 28) | (cell & 0x0FFFFFFFu);
    s->k = 0;
    s->umode = umode;
}

static inline double stream_draw(orc_stream *s) {
    const uint32_t half = s->k & 1u;
    if (half == 0) {
        s->ctr[0] = s->k >> 1;
        orc_philox4x32_10(s->ctr, s->key, s->buf);
    }
    ++s->k;
    const uint64_t w = ((uint64_t)s->buf[2 * half + 1] << 32) | s->buf[2 * half];
    if (s->umode == ORC_U24) {
        uint64_t m = w >> 40;
        if (m == 0) m = 1;
        return (double)m * 0x1p-24;
    }
    uint64_t m = w >> 11;
    if (m == 0) m = 1;
    return (double)m * 0x1p-53;
}

void orc_uniforms(uint64_t seed, uint32_t cell, uint32_t cru, uint64_t step, uint32_t stream,
                  int umode, uint32_t k0, int n, double *out) {
    orc_stream s;
    stream_open(&s, seed, cell, cru, step, stream, umode);
    for (uint32_t k = 0; k < k0; ++k) (void)stream_draw(&s);
    for (int i = 0; i < n; ++i) out[i] = stream_draw(&s);
}

/* sample_binomial, common.hpp:37-47 */
static inline int sample_binomial(orc_stream *s, double p, int N) {
    int X = 0;
    for (int i = 0; i < N; i++) {
        const double u = stream_draw(s);
        if (u < p) X++;
    }
    return X;
}

/* sample_weights, common.hpp:49-59 */
static inline int sample_weights(orc_stream *s, const double *w, double total, int size) {
    const double u = stream_draw(s) * total;
    double cum = w[0];
    int i = 0;
    while (cum < u && i < (size - 1)) {
        ++i;
        cum += w[i];
    }
    return i;
}

/* ------------------------------------------------------------------------------------------ */
/* per-CRU SSA (SSA.hpp:15-43, SSA.tpp)                                                        */
/* ------------------------------------------------------------------------------------------ */

typedef struct orc_cru {
    int LCC[4], LCCi[4], RyR[24], ClCh[4];
    double open_RyR[4];
    double CaSS[4], CaJSR, JLCC[4], Jrel[4], Jxfer[4], Jiss[4], Jtr;
    double LCC_rates[12], LCCi_rates[4], RyR_rates[48], ClCh_rates[4], subunit_rates[4];
} orc_cru;

/* update_LCC_rates, GW_utils.tpp:118-186 */
static void lcc_rates(orc_cru *s, int idx, const orc_params *p, const orc_consts *c) {
    double *r = s->LCC_rates + 3 * idx;
    const double x = s->CaSS[idx];
    switch (s->LCC[idx]) {
    case 1: r[0] = 4 * c->alphaLCC; r[1] = c->gamma0 * x; r[2] = 0; break;
    case 2: r[0] = c->betaLCC; r[1] = 3 * c->alphaLCC; r[2] = c->gamma0a * x; break;
    case 3: r[0] = 2 * c->betaLCC; r[1] = 2 * c->alphaLCC; r[2] = c->gamma0a2 * x; break;
    case 4: r[0] = 3 * c->betaLCC; r[1] = c->alphaLCC; r[2] = c->gamma0a3 * x; break;
    case 5: r[0] = 4 * c->betaLCC; r[1] = p->f; r[2] = c->gamma0a4 * x; break;
    case 6: r[0] = p->g; r[1] = 0; r[2] = 0; break;
    case 7: r[0] = c->omega; r[1] = 4 * c->alphaLCC * c->a; r[2] = 0; break;
    case 8: r[0] = c->omega_b; r[1] = c->betaLCC * c->binv; r[2] = 3 * c->alphaLCC * c->a; break;
    case 9: r[0] = c->omega_b2; r[1] = 2 * c->betaLCC * c->binv; r[2] = 2 * c->alphaLCC * c->a; break;
    case 10: r[0] = c->omega_b3; r[1] = 3 * c->betaLCC * c->binv; r[2] = c->alphaLCC * c->a; break;
    case 11: r[0] = c->omega_b4; r[1] = 4 * c->betaLCC * c->binv; r[2] = p->f1; break;
    case 12: r[0] = p->g1; r[1] = 0; r[2] = 0; break;
    default: break;
    }
    s->subunit_rates[idx] += (r[0] + r[1] + r[2]);
}

/* update_LCC_inactivation_rates, GW_utils.hpp:378-383 */
static void lcci_rates(orc_cru *s, int idx, const orc_consts *c) {
    s->LCCi_rates[idx] = (s->LCCi[idx] == 0) ? c->yinfLCC / c->tauLCC : (1.0 - c->yinfLCC) / c->tauLCC;
    s->subunit_rates[idx] += s->LCCi_rates[idx];
}

/* update_RyR_rates, GW_utils.tpp:222-255 */
static void ryr_rates(orc_cru *s, int idx, const orc_params *p) {
    const int *R = s->RyR + 6 * idx;
    double *r = s->RyR_rates + 12 * idx;
    const double x = s->CaSS[idx];
    const double x2 = x * x;
    const double eq56 = p->k65 / (p->k56 * x2 + p->k65);
    const double tau34 = 1.0 / (p->k34 * x2 + p->k43);
    r[0] = R[0] * p->k12 * x2;
    r[1] = R[1] * p->k23 * x2;
    r[2] = R[1] * p->k25 * x2;
    r[3] = x > 3.685e-2 ? 0 : R[2] * p->k34 * x2;
    r[4] = x > 3.685e-2 ? (R[2] + R[3]) * p->k45 * p->k34 * x2 * tau34 : R[3] * p->k45;
    r[5] = x > 1.15e-4 ? 0 : R[4] * p->k56 * x2;
    r[6] = R[1] * p->k21;
    r[7] = x > 3.685e-2 ? (R[2] + R[3]) * p->k32 * p->k43 * tau34 : R[2] * p->k32;
    r[8] = x > 3.685e-2 ? 0 : R[3] * p->k43;
    r[9] = x > 1.15e-4 ? (R[4] + R[5]) * p->k52 * eq56 : R[4] * p->k52;
    r[10] = x > 1.15e-4 ? (R[4] + R[5]) * p->k54 * x2 * eq56 : R[4] * p->k54 * x2;
    r[11] = x > 1.15e-4 ? 0 : R[5] * p->k65;
    for (int k = 0; k < 12; k++) s->subunit_rates[idx] += r[k];
}

/* update_ClCh_rates, GW_utils.hpp:386-391 */
static void clch_rates(orc_cru *s, int idx, const orc_params *p) {
    s->ClCh_rates[idx] = (s->ClCh[idx] == 0) ? p->kfClCh * s->CaSS[idx] : p->kbClCh;
    s->subunit_rates[idx] += s->ClCh_rates[idx];
}

/* update_rates, SSA.tpp:48-56 */
static void update_rates(orc_cru *s, const orc_params *p, const orc_consts *c) {
    for (int j = 0; j < 4; j++) {
        s->subunit_rates[j] = 0;
        lcc_rates(s, j, p, c);
        lcci_rates(s, j, c);
        ryr_rates(s, j, p);
        clch_rates(s, j, p);
    }
}

/* update_fluxes, SSA.tpp:37-45 */
static void update_fluxes(orc_cru *s, double Cai, double CaNSR, const orc_params *p) {
    s->Jtr = p->rtr * (CaNSR - s->CaJSR);
    s->Jiss[0] = p->riss * (s->CaSS[1] + s->CaSS[3] - 2 * s->CaSS[0]);
    s->Jiss[1] = p->riss * (s->CaSS[2] + s->CaSS[0] - 2 * s->CaSS[1]);
    s->Jiss[2] = p->riss * (s->CaSS[3] + s->CaSS[1] - 2 * s->CaSS[2]);
    s->Jiss[3] = p->riss * (s->CaSS[0] + s->CaSS[2] - 2 * s->CaSS[3]);
    for (int j = 0; j < 4; j++) s->Jxfer[j] = p->rxfer * (s->CaSS[j] - Cai);
}

/* sample_RyR56 / sample_RyR34, SSA.tpp:59-84 */
static void resplit(orc_stream *rs, orc_cru *s, int idx, int lo, double kdown, double kup) {
    const int n = s->RyR[lo + 6 * idx] + s->RyR[lo + 1 + 6 * idx];
    if (n > 0) {
        const double pr = kdown / (kdown + kup * sq(s->CaSS[idx]));
        s->RyR[lo + 6 * idx] = sample_binomial(rs, pr, n);
        s->RyR[lo + 1 + 6 * idx] = n - s->RyR[lo + 6 * idx];
    } else {
        s->RyR[lo + 6 * idx] = 0;
        s->RyR[lo + 1 + 6 * idx] = 0;
    }
}

/* update_CaSS, SSA.tpp:87-99 */
static void update_CaSS(orc_stream *rs, orc_cru *s, double dt, const orc_params *p,
                        const orc_consts *c) {
    for (int j = 0; j < 4; j++) {
        const double betaSS = 1.0 / (1 + (c->BSR_const / sq(p->KBSR + s->CaSS[j])) +
                                     (c->BSL_const / sq(p->KBSL + s->CaSS[j])));
        const double dCaSS = dt * (s->JLCC[j] + s->Jrel[j] - s->Jxfer[j] + s->Jiss[j]) * betaSS;
        const double tmp = s->CaSS[j] + dCaSS;
        if (s->CaSS[j] > 1.15e-4 && tmp <= 1.15e-4)
            resplit(rs, s, j, 4, p->k65, p->k56);
        else if (s->CaSS[j] > 0.03685 && tmp <= 0.03685)
            resplit(rs, s, j, 2, p->k43, p->k34);
        s->CaSS[j] = tmp;
    }
}

/* update_CaJSR, SSA.hpp:68-71 */
static void update_CaJSR(orc_cru *s, double dt, const orc_params *p, const orc_consts *c) {
    const double betaJSR = 1.0 / (1 + c->CSQN_const / sq(p->KCSQN + s->CaJSR));
    s->CaJSR += (dt * betaJSR *
                 (s->Jtr - c->VSS_VJSR * (s->Jrel[0] + s->Jrel[1] + s->Jrel[2] + s->Jrel[3])));
}

static inline double jlcc_open(const orc_cru *s, int j, const orc_consts *c) {
    return c->JLCC_multiplier * (c->Cao_scaled - c->JLCC_exp * s->CaSS[j]);
}

/* sample_LCC, SSA.tpp:103-197: transition table by state, JLCC on entering/leaving 6 and 12. */
static void sample_LCC(orc_stream *rs, orc_cru *s, double sum, int j, const orc_consts *c) {
    static const signed char next[13][3] = {
        {0, 0, 0},  {2, 7, 7},   {1, 3, 8},   {2, 4, 9},  {3, 5, 10},  {4, 6, 11}, {5, 5, 5},
        {1, 8, 8},  {2, 7, 9},   {3, 8, 10},  {4, 9, 11}, {5, 10, 12}, {11, 11, 11}};
    const int tr = sample_weights(rs, s->LCC_rates + 3 * j, sum, 3);
    const int from = s->LCC[j];
    if (from < 1 || from > 12) return;
    const int to = next[from][tr];
    s->LCC[j] = to;
    if ((from == 5 && to == 6) || (from == 11 && to == 12))
        s->JLCC[j] = (s->LCCi[j] == 1) ? jlcc_open(s, j, c) : 0;
    else if (from == 6 || from == 12)
        s->JLCC[j] = 0;
}

/* sample_RyR, SSA.tpp:200-259: (from, to) state of each of the 12 transitions, open-count delta. */
static void sample_RyR(orc_stream *rs, orc_cru *s, double sum, int j, const orc_params *p) {
    static const signed char from[12] = {0, 1, 1, 2, 3, 4, 1, 2, 3, 4, 4, 5};
    static const signed char to[12] = {1, 2, 4, 3, 4, 5, 0, 1, 2, 1, 3, 4};
    static const signed char dopen[12] = {0, 1, 0, 0, -1, 0, 0, -1, 0, 0, 1, 0};
    const int tr = sample_weights(rs, s->RyR_rates + 12 * j, sum, 12);
    --s->RyR[6 * j + from[tr]];
    ++s->RyR[6 * j + to[tr]];
    s->open_RyR[j] += dopen[tr];
    s->Jrel[j] = p->rRyR * s->open_RyR[j] * (s->CaJSR - s->CaSS[j]);
}

/* sample_new_state, SSA.tpp:262-283 */
static void sample_new_state(orc_stream *rs, orc_cru *s, int j, const orc_params *p,
                             const orc_consts *c) {
    const double sub = s->subunit_rates[j];
    const double sum_LCC = s->LCC_rates[3 * j] + s->LCC_rates[3 * j + 1] + s->LCC_rates[3 * j + 2];
    const double inact = s->LCCi_rates[j];
    const double clch = s->ClCh_rates[j];
    const double sum_RyR = sub - (sum_LCC + inact + clch);
    const double u = stream_draw(rs) * sub;
    if (u < sum_LCC) {
        sample_LCC(rs, s, sum_LCC, j, c);
    } else if (u < (sum_LCC + inact)) {
        s->LCCi[j] = 1 - s->LCCi[j];
        if (s->LCCi[j] == 0)
            s->JLCC[j] = 0;
        else if ((s->LCC[j] == 6) || (s->LCC[j] == 12))
            s->JLCC[j] = jlcc_open(s, j, c);
    } else if (u < (sum_LCC + inact + sum_RyR)) {
        sample_RyR(rs, s, sum_RyR, j, p);
    } else {
        s->ClCh[j] = 1 - s->ClCh[j];
    }
}

/* SSA_single_CRU, SSA.tpp:286-310.  Returns the number of jumps taken. */
static int64_t ssa_single_cru(orc_stream *rs, orc_cru *s, double Cai, double CaNSR, double dt,
                              const orc_params *p, const orc_consts *c) {
    double t = 0, jump_t = 0, total;
    int64_t events = 0;
    for (;;) {
        update_fluxes(s, Cai, CaNSR, p);
        update_rates(s, p, c);
        total = s->subunit_rates[0] + s->subunit_rates[1] + s->subunit_rates[2] + s->subunit_rates[3];
        jump_t = -log(stream_draw(rs)) / total;
        if (t + jump_t < dt) {
            update_CaSS(rs, s, jump_t, p, c);
            update_CaJSR(s, jump_t, p, c);
        } else {
            update_CaSS(rs, s, dt - t, p, c);
            update_CaJSR(s, dt - t, p, c);
            break;
        }
        t += jump_t;
        const int sub = sample_weights(rs, s->subunit_rates, total, 4);
        sample_new_state(rs, s, sub, p, c);
        ++events;
    }
    return events;
}

/* ------------------------------------------------------------------------------------------ */
/* model (GW.hpp:45-124, GW.tpp)                                                               */
/* ------------------------------------------------------------------------------------------ */

struct orc_model {
    int n;
    orc_params p;
    orc_consts c;
    orc_globals g, dg;
    orc_currents cur;
    double *CaSS, *CaJSR, *JLCC, *Jxfer, *Jtr;
    int *LCC, *LCCi, *RyR, *ClCh;
    double QKr[5][5], QKv14[10][10], QKv43[10][10];
    double Istim;
    uint64_t seed, step;
    uint32_t cell;
    int umode;
    int64_t events;
};

/* GW_model ctor, GW.hpp:104-113.  The reference's ctor first draws a random CRUState and computes
 * JLCC/Jxfer/Jtr from it and the default GlobalState; set_initial_value then overwrites the
 * state but not those fluxes.  Random initial LCC states are 1, 2 or 7, so the initial JLCC is 0;
 * initial CaSS/CaJSR are the constants 1.45370e-4 / 0.908408 (GW_utils.tpp:212-213). */
orc_model *orc_create(const orc_params *p, int nCRU, uint64_t seed, uint32_t cell, int umode) {
    orc_model *m = (orc_model *)calloc(1, sizeof *m);
    if (!m) return NULL;
    m->n = nCRU;
    m->p = *p;
    m->seed = seed;
    m->cell = cell;
    m->umode = umode;
    orc_constants(p, nCRU, &m->c);
    orc_globals_default(&m->g);
    const size_t n = (size_t)nCRU;
    m->CaSS = (double *)calloc(4 * n, sizeof(double));
    m->CaJSR = (double *)calloc(n, sizeof(double));
    m->JLCC = (double *)calloc(4 * n, sizeof(double));
    m->Jxfer = (double *)calloc(4 * n, sizeof(double));
    m->Jtr = (double *)calloc(n, sizeof(double));
    m->LCC = (int *)calloc(4 * n, sizeof(int));
    m->LCCi = (int *)calloc(4 * n, sizeof(int));
    m->RyR = (int *)calloc(24 * n, sizeof(int));
    m->ClCh = (int *)calloc(4 * n, sizeof(int));
    for (size_t i = 0; i < 4 * n; ++i) m->CaSS[i] = 1.45370e-4;
    for (size_t i = 0; i < n; ++i) m->CaJSR[i] = 0.908408;
    for (size_t i = 0; i < 4 * n; ++i) m->LCC[i] = 1;
    /* initialise_Jxfer / initialise_Jtr (GW.hpp:73-74) from the default GlobalState. */
    for (size_t i = 0; i < 4 * n; ++i) m->Jxfer[i] = p->rxfer * (m->CaSS[i] - m->g.Cai);
    for (size_t i = 0; i < n; ++i) m->Jtr[i] = p->rtr * (m->g.CaNSR - m->CaJSR[i]);
    /* initialise_QKr (GW.hpp:75) */
    m->QKr[1][2] = p->Kf;
    m->QKr[2][1] = p->Kb;
    return m;
}

void orc_destroy(orc_model *m) {
    if (!m) return;
    free(m->CaSS); free(m->CaJSR); free(m->JLCC); free(m->Jxfer); free(m->Jtr);
    free(m->LCC); free(m->LCCi); free(m->RyR); free(m->ClCh);
    free(m);
}

int orc_ncru(const orc_model *m) { return m->n; }
void orc_set_globals(orc_model *m, const orc_globals *g) { m->g = *g; }
void orc_get_globals(const orc_model *m, orc_globals *g) { *g = m->g; }
void orc_get_consts(const orc_model *m, orc_consts *c) { *c = m->c; }
void orc_get_currents(const orc_model *m, orc_currents *cur) { *cur = m->cur; }
void orc_set_step(orc_model *m, uint64_t step) { m->step = step; }
uint64_t orc_get_step(const orc_model *m) { return m->step; }
int64_t orc_event_count(const orc_model *m) { return m->events; }

void orc_set_crus(orc_model *m, const double *CaSS, const double *CaJSR, const int *LCC,
                  const int *LCCi, const int *RyR, const int *ClCh) {
    const size_t n = (size_t)m->n;
    if (CaSS) memcpy(m->CaSS, CaSS, 4 * n * sizeof(double));
    if (CaJSR) memcpy(m->CaJSR, CaJSR, n * sizeof(double));
    if (LCC) memcpy(m->LCC, LCC, 4 * n * sizeof(int));
    if (LCCi) memcpy(m->LCCi, LCCi, 4 * n * sizeof(int));
    if (RyR) memcpy(m->RyR, RyR, 24 * n * sizeof(int));
    if (ClCh) memcpy(m->ClCh, ClCh, 4 * n * sizeof(int));
}

void orc_get_crus(const orc_model *m, double *CaSS, double *CaJSR, int *LCC, int *LCCi, int *RyR,
                  int *ClCh) {
    const size_t n = (size_t)m->n;
    if (CaSS) memcpy(CaSS, m->CaSS, 4 * n * sizeof(double));
    if (CaJSR) memcpy(CaJSR, m->CaJSR, n * sizeof(double));
    if (LCC) memcpy(LCC, m->LCC, 4 * n * sizeof(int));
    if (LCCi) memcpy(LCCi, m->LCCi, 4 * n * sizeof(int));
    if (RyR) memcpy(RyR, m->RyR, 24 * n * sizeof(int));
    if (ClCh) memcpy(ClCh, m->ClCh, 4 * n * sizeof(int));
}

void orc_set_fluxes(orc_model *m, const double *JLCC, const double *Jxfer, const double *Jtr) {
    const size_t n = (size_t)m->n;
    if (JLCC) memcpy(m->JLCC, JLCC, 4 * n * sizeof(double));
    if (Jxfer) memcpy(m->Jxfer, Jxfer, 4 * n * sizeof(double));
    if (Jtr) memcpy(m->Jtr, Jtr, n * sizeof(double));
}

void orc_get_fluxes(const orc_model *m, double *JLCC, double *Jxfer, double *Jtr) {
    const size_t n = (size_t)m->n;
    if (JLCC) memcpy(JLCC, m->JLCC, 4 * n * sizeof(double));
    if (Jxfer) memcpy(Jxfer, m->Jxfer, 4 * n * sizeof(double));
    if (Jtr) memcpy(Jtr, m->Jtr, n * sizeof(double));
}

/* Random initial CRU state, GW_utils.tpp:5-64 (weights also at ms_experiment.py:51-63), drawn per
 * CRU from stream INIT in the order LCC[0..3], LCC_inactivation[0..3], RyR[0..3]x5, ClCh[0..3]. */
void orc_sample_initial_crus(orc_model *m) {
    static const double wl[3] = {0.958, 0.038, 0.004};
    static const double wi[2] = {0.9425, 0.0575};
    static const double wr[3] = {0.609, 0.5 * 0.391, 0.5 * 0.391};
    static const double wc[2] = {0.998, 0.002};
    static const int lcc_of[3] = {1, 2, 7};
    static const int ryr_of[3] = {0, 4, 5};
    for (int i = 0; i < m->n; ++i) {
        orc_stream s;
        stream_open(&s, m->seed, m->cell, (uint32_t)i, 0, ORC_STREAM_INIT, m->umode);
        for (int j = 0; j < 4; ++j) m->LCC[4 * i + j] = lcc_of[sample_weights(&s, wl, 1.0, 3)];
        for (int j = 0; j < 4; ++j) m->LCCi[4 * i + j] = sample_weights(&s, wi, 1.0, 2) == 0 ? 1 : 0;
        for (int j = 0; j < 4; ++j) {
            for (int k = 0; k < 6; ++k) m->RyR[24 * i + 6 * j + k] = 0;
            for (int k = 0; k < 5; ++k) ++m->RyR[24 * i + 6 * j + ryr_of[sample_weights(&s, wr, 1.0, 3)]];
        }
        for (int j = 0; j < 4; ++j) m->ClCh[4 * i + j] = sample_weights(&s, wc, 1.0, 2);
        for (int j = 0; j < 4; ++j) m->CaSS[4 * i + j] = 1.45370e-4;
        m->CaJSR[i] = 0.908408;
    }
}

/* update_QKr, GW.tpp:26-44 */
static void update_QKr(orc_model *m) {
    double (*Q)[5] = m->QKr;
    const double V = m->g.V;
    Q[0][1] = 0.0069 * exp(0.0272 * V);
    Q[0][0] = -Q[0][1];
    Q[1][0] = 0.0227 * exp(-0.0431 * V);
    Q[1][1] = -(Q[1][0] + Q[1][2]);
    Q[2][3] = 0.0218 * exp(0.0262 * V);
    Q[2][4] = 1.29e-5 * exp(2.71e-6 * V);
    Q[2][2] = -(Q[2][1] + Q[2][3] + Q[2][4]);
    Q[3][2] = 0.0009 * exp(-0.0269 * V);
    Q[3][4] = 0.0622 * exp(0.0120 * V);
    Q[3][3] = -(Q[3][2] + Q[3][4]);
    Q[4][3] = 0.0059 * exp(-0.0443 * V);
    Q[4][2] = Q[3][2] * Q[4][3] * Q[2][4] / (Q[2][3] * Q[3][4]);
    Q[4][4] = -(Q[4][2] + Q[4][3]);
}

/* The 10-state Kv1.4 / Kv4.3 generator; update_QKv, GW.tpp:65-123 (one channel per call). */
static void fill_QKv(double Q[10][10], double aa, double ai, double ba, double bi, double f1,
                     double f2, double f3, double f4, double b1, double b2, double b3, double b4) {
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

static void update_QKv(orc_model *m) {
    const orc_params *p = &m->p;
    const double V = m->g.V;
    const double aa14 = p->alphaa0Kv14 * exp(p->aaKv14 * V);
    const double aa43 = p->alphaa0Kv43 * exp(p->aaKv43 * V);
    const double ai14 = p->alphai0Kv14 * exp(-p->aiKv14 * V);
    const double ai43 = p->alphai0Kv43 * exp(-p->aiKv43 * V);
    const double ba14 = p->betaa0Kv14 * exp(-p->baKv14 * V);
    const double ba43 = p->betaa0Kv43 * exp(-p->baKv43 * V);
    const double bi14 = p->betai0Kv14 * exp(p->biKv14 * V);
    const double bi43 = p->betai0Kv43 * exp(p->biKv43 * V);
    fill_QKv(m->QKv14, aa14, ai14, ba14, bi14, p->f1Kv14, p->f2Kv14, p->f3Kv14, p->f4Kv14,
             p->b1Kv14, p->b2Kv14, p->b3Kv14, p->b4Kv14);
    fill_QKv(m->QKv43, aa43, ai43, ba43, bi43, p->f1Kv43, p->f2Kv43, p->f3Kv43, p->f4Kv43,
             p->b1Kv43, p->b2Kv43, p->b3Kv43, p->b4Kv43);
}

/* common::Nernst, common.hpp:70-77 (the reference exits on a non-positive argument). */
static double nernst(double Xi, double Xo, double RT_F, double valence) {
    if (Xi <= 0.0 || Xo <= 0.0) return NAN;
    return log(Xo / Xi) * RT_F / valence;
}

/* update_V_and_concentration_derivatives, GW.tpp:171-212 (currents: common.hpp:89-168,
 * GW_utils.hpp:273-355).  ECa uses Ki/Ko with valence 2, as in the reference (GW.tpp:176). */
static void update_V_and_conc(orc_model *m, double dt) {
    const orc_params *p = &m->p;
    orc_consts *c = &m->c;
    const orc_globals *g = &m->g;
    orc_currents *I = &m->cur;
    orc_globals *d = &m->dg;
    const double V = g->V;
    c->ENa = nernst(g->Nai, p->Nao, c->RT_F, 1.0);
    c->EK = nernst(g->Ki, p->Ko, c->RT_F, 1.0);
    c->ECa = nernst(g->Ki, p->Ko, c->RT_F, 2.0);

    I->INa = p->GNa * cube(g->m) * g->h * g->j * (V - c->ENa);
    I->INab = p->GNab * (V - c->ENa);
    {
        const double e1 = exp(p->eta * c->VF_RT);
        const double e2 = e1 * c->expmVF_RT;
        I->INaCa = c->INaCa_const * (e1 * cube(g->Nai) * p->Cao - e2 * c->Nao3 * g->Cai) /
                   (1.0 + p->ksat * e2);
    }
    {
        const double fNaK = 1.0 / (1.0 + 0.1245 * exp(-0.1 * c->VF_RT) + 0.0365 * c->sigma * c->expmVF_RT);
        I->INaK = c->INaK_const * fNaK / (1.0 + pow(p->KmNai / g->Nai, 1.5));
    }
    {
        const double RKr = 1.0 / (1.0 + 1.4945 * exp(0.0446 * V));
        I->IKr = p->GKr * c->sqrtKo * RKr * g->Kr[3] * (V - c->EK) * 0.5;
    }
    {
        const double EKs = log((p->Ko + 0.01833 * p->Nao) / (g->Ki + 0.01833 * g->Nai)) * c->RT_F;
        I->IKs = p->GKs * sq(g->xKs) * (V - EKs);
    }
    double IKv14, IKv43;
    {
        const double e = c->expmVF_RT;
        const double mm = (c->PKv14_Csc) * (FARADAY * c->VF_RT) * g->Kv14[4] / (1 - e);
        IKv14 = mm * ((g->Ki - p->Ko * e) + 0.02 * (g->Nai - p->Nao * e)) * 1.0e9;
    }
    IKv43 = p->GKv43 * g->Kv43[4] * (V - c->EK);
    I->Ito1 = IKv14 + IKv43;
    {
        long clsum = 0;
        for (int i = 0; i < 4 * m->n; ++i) clsum += m->ClCh[i];
        I->Ito2 = (double)clsum * c->Ito2_const * c->VF_RT * (p->Clcyto * c->expmVF_RT - p->Clo) /
                  (c->expmVF_RT - 1.0);
    }
    {
        const double K1inf = 1.0 / (2.0 + exp(1.5 * (V - c->EK) * c->F_RT));
        I->IK1 = p->GK1 * K1inf * c->IK1_const * (V - c->EK);
    }
    {
        const double Kp = 1. / (1. + exp((7.488 - V) / 5.98));
        I->IKp = p->GKp * Kp * (V - c->EK);
    }
    {
        double s = 0;
        for (int i = 0; i < 4 * m->n; ++i) s += m->JLCC[i];
        I->ICaL = s * c->ICaL_const;
    }
    I->ICab = p->GCab * (V - c->ECa);
    I->IpCa = p->IpCamax * (g->Cai / (p->KmpCa + g->Cai));
    {
        const double f = pow(g->Cai / p->Kmf, p->Hf);
        const double r = pow(g->CaNSR / p->Kmr, p->Hr);
        I->Jup = (p->Vmaxf * f - p->Vmaxr * r) / (1.0 + f + r);
    }
    {
        double s = 0;
        for (int i = 0; i < m->n; ++i) s += m->Jtr[i];
        I->Jtr_tot = s * c->CRU_factor;
        s = 0;
        for (int i = 0; i < 4 * m->n; ++i) s += m->Jxfer[i];
        I->Jxfer_tot = s * c->CRU_factor;
    }
    c->beta_cyto = 1.0 / (1.0 + c->CMDN_const / sq(p->KCMDN + g->Cai));

    d->CaLTRPN = p->kLTRPNp * g->Cai * (p->LTRPNtot - g->CaLTRPN) - p->kLTRPNm * g->CaLTRPN;
    d->CaHTRPN = p->kHTRPNp * g->Cai * (p->HTRPNtot - g->CaHTRPN) - p->kHTRPNm * g->CaHTRPN;

    d->Nai = -dt * c->CSA_FVcyto * (I->INa + I->INab + 3 * I->INaCa + 3 * I->INaK);
    d->Ki = -dt * c->CSA_FVcyto * (I->IKr + I->IKs + I->Ito1 + I->IK1 + I->IKp - 2 * I->INaK);
    d->Cai = dt * c->beta_cyto *
             (-0.5 * c->CSA_FVcyto * (I->ICab + I->IpCa - 2 * I->INaCa) +
              c->VSS_Vcyto * I->Jxfer_tot - I->Jup - (d->CaLTRPN + d->CaHTRPN));
    d->CaNSR = dt * (c->Vcyto_VNSR * I->Jup - c->VJSR_VNSR * I->Jtr_tot);
    d->CaLTRPN *= dt;
    d->CaHTRPN *= dt;
    d->V = dt * (m->Istim - (I->INa + I->ICaL + I->IKr + I->IKs + I->Ito1 + I->IK1 + I->IKp +
                             I->Ito2 + I->INaK + I->INaCa + I->IpCa + I->ICab + I->INab));
}

/* update_gate_derivatives, GW.tpp:163-168 (rates: common.hpp:175-218, GW_utils.hpp:358-362) */
static void update_gates(orc_model *m, double dt) {
    const double V = m->g.V;
    orc_globals *d = &m->dg;
    const orc_globals *g = &m->g;
    const double am = (V == -47.13) ? 3.2 : 0.32 * (V + 47.13) / (1.0 - exp(-0.1 * (V + 47.13)));
    const double bm = 0.08 * exp(-V / 11.0);
    const double ah = (V >= -40.0) ? 0.0 : 0.135 * exp(-(V + 80.0) / 6.8);
    const double bh = (V >= -40.0) ? 1.0 / (0.13 * (1.0 + exp(-(V + 10.66) / 11.1)))
                                   : 3.56 * exp(0.079 * V) + 3.1e5 * exp(0.35 * V);
    const double aj = (V >= -40.0) ? 0.0
                                   : (-127140.0 * exp(0.2444 * V) - 3.474e-5 * exp(-0.04391 * V)) *
                                         (V + 37.78) / (1.0 + exp(0.311 * (V + 79.23)));
    const double bj = (V >= -40.0) ? 0.3 * exp(-2.535e-7 * V) / (1.0 + exp(-0.1 * (V + 32.0)))
                                   : 0.1212 * exp(-0.01052 * V) / (1.0 + exp(-0.1378 * (V + 40.14)));
    const double xinf = 1.0 / (1.0 + exp(-(V - 24.7) / 13.6));
    const double tinv = 0.0000719 * (V - 10.0) / (1.0 - exp(-0.148 * (V - 10.0))) +
                        0.000131 * (V - 10.0) / (exp(0.0687 * (V - 10.0)) - 1.0);
    d->m = dt * (am * (1.0 - g->m) - bm * g->m);
    d->h = dt * (ah * (1.0 - g->h) - bh * g->h);
    d->j = dt * (aj * (1.0 - g->j) - bj * g->j);
    d->xKs = dt * (xinf - g->xKs) * tinv;
}

/* update_Kr_derivatives, GW.tpp:127-133 */
static void update_Kr(orc_model *m, double dt) {
    double (*Q)[5] = m->QKr;
    const double *x = m->g.Kr;
    double *d = m->dg.Kr;
    d[0] = dt * (Q[1][0] * x[1] + Q[0][0] * x[0]);
    d[1] = dt * (Q[0][1] * x[0] + Q[2][1] * x[2] + Q[1][1] * x[1]);
    d[2] = dt * (Q[1][2] * x[1] + Q[3][2] * x[3] + Q[4][2] * x[4] + Q[2][2] * x[2]);
    d[3] = dt * (Q[2][3] * x[2] + Q[4][3] * x[4] + Q[3][3] * x[3]);
    d[4] = dt * (Q[2][4] * x[2] + Q[3][4] * x[3] + Q[4][4] * x[4]);
}

/* update_Kv_derivatives, GW.tpp:136-160 (same stencil for both channels) */
static void kv_deriv(double Q[10][10], const double *x, double *d, double dt) {
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

/* GW_model::SSA, GW.tpp:215-234: gather, SSA_single_CRU, scatter, per CRU. */
static void ssa_all(orc_model *m, double dt) {
    orc_ssa_step_constants(&m->c, m->g.V);
    const double Cai = m->g.Cai, CaNSR = m->g.CaNSR;
    int64_t events = 0;
#pragma omp parallel for schedule(static) reduction(+ : events)
    for (int i = 0; i < m->n; i++) {
        orc_cru s;
        memset(&s, 0, sizeof s);
        orc_stream rs;
        stream_open(&rs, m->seed, m->cell, (uint32_t)i, m->step, ORC_STREAM_SSA, m->umode);
        /* copy_from_CRUState, SSA.tpp:10-33 */
        for (int j = 0; j < 4; j++) {
            for (int k = 0; k < 6; k++) s.RyR[6 * j + k] = m->RyR[24 * i + 6 * j + k];
            s.LCC[j] = m->LCC[4 * i + j];
            s.LCCi[j] = m->LCCi[4 * i + j];
            s.ClCh[j] = m->ClCh[4 * i + j];
            s.open_RyR[j] = (double)(m->RyR[24 * i + 6 * j + 2] + m->RyR[24 * i + 6 * j + 3]);
            s.CaSS[j] = m->CaSS[4 * i + j];
            s.JLCC[j] = m->JLCC[4 * i + j];
            s.Jrel[j] = m->p.rRyR * s.open_RyR[j] * (m->CaJSR[i] - s.CaSS[j]);
        }
        s.CaJSR = m->CaJSR[i];
        events += ssa_single_cru(&rs, &s, Cai, CaNSR, dt, &m->p, &m->c);
        /* update_CRUstate_from_temp, GW.tpp:48-62 */
        for (int j = 0; j < 4; j++) {
            m->LCC[4 * i + j] = s.LCC[j];
            m->LCCi[4 * i + j] = s.LCCi[j];
            for (int k = 0; k < 6; k++) m->RyR[24 * i + 6 * j + k] = s.RyR[6 * j + k];
            m->ClCh[4 * i + j] = s.ClCh[j];
            m->CaSS[4 * i + j] = s.CaSS[j];
            m->JLCC[4 * i + j] = s.JLCC[j];
            m->Jxfer[4 * i + j] = s.Jxfer[j];
        }
        m->CaJSR[i] = s.CaJSR;
        m->Jtr[i] = s.Jtr;
    }
    m->events += events;
}

/* euler_step, GW.tpp:237-272 */
void orc_euler_step(orc_model *m, double dt, double Istim) {
    m->Istim = Istim;
    m->c.VF_RT = m->g.V * m->c.F_RT;
    m->c.expmVF_RT = exp(-m->c.VF_RT);
    update_QKr(m);
    update_QKv(m);
    update_V_and_conc(m, dt);
    update_gates(m, dt);
    update_Kr(m, dt);
    kv_deriv(m->QKv14, m->g.Kv14, m->dg.Kv14, dt);
    kv_deriv(m->QKv43, m->g.Kv43, m->dg.Kv43, dt);
    ssa_all(m, dt);
    orc_globals *g = &m->g;
    const orc_globals *d = &m->dg;
    g->V += d->V;
    g->Nai += d->Nai;
    g->Ki += d->Ki;
    g->Cai += d->Cai;
    g->CaNSR += d->CaNSR;
    g->CaLTRPN += d->CaLTRPN;
    g->CaHTRPN += d->CaHTRPN;
    g->m += d->m;
    g->h += d->h;
    g->j += d->j;
    g->xKs += d->xKs;
    for (int k = 0; k < 5; k++) g->Kr[k] += d->Kr[k];
    for (int k = 0; k < 10; k++) {
        g->Kv14[k] += d->Kv14[k];
        g->Kv43[k] += d->Kv43[k];
    }
    ++m->step;
}

/* run<PRNG>, pyGW.hpp:102-122 (time accumulated by t += dt; record after step i when
 * i % record_every == 0). */
int64_t orc_run(orc_model *m, double dt, int64_t num_steps, const double *Istim, int record_every,
                int64_t max_records, double *rec_t, orc_globals *rec_globals) {
    double t = 0.0;
    int64_t counter = 0;
    for (int64_t i = 0; i < num_steps; ++i) {
        orc_euler_step(m, dt, Istim ? Istim[i] : 0.0);
        t += dt;
        if (record_every > 0 && i % record_every == 0) {
            if (counter < max_records) {
                if (rec_t) rec_t[counter] = t;
                if (rec_globals) rec_globals[counter] = m->g;
            }
            ++counter;
        }
    }
    return counter < max_records ? counter : max_records;
}

/* run<PRNG> with record_state (pyGW.hpp:56-122): the same loop as orc_run, and at each record the
 * CRU arrays as well (record_state copies every CRU array, pyGW.hpp:84-98).  Any record pointer
 * may be NULL.  Returns the number of records the reference's loop makes (ceil(num_steps /
 * record_every)); only the first max_records of them are stored. */
int64_t orc_run_record(orc_model *m, double dt, int64_t num_steps, const double *Istim,
                       int record_every, int64_t max_records, double *rec_t,
                       orc_globals *rec_globals, double *rec_CaSS, double *rec_CaJSR,
                       int *rec_LCC, int *rec_LCCi, int *rec_RyR, int *rec_ClCh) {
    const size_t n = (size_t)m->n;
    double t = 0.0;
    int64_t counter = 0;
    for (int64_t i = 0; i < num_steps; ++i) {
        orc_euler_step(m, dt, Istim ? Istim[i] : 0.0);
        t += dt;
        if (record_every > 0 && i % record_every == 0) {
            if (counter < max_records) {
                const size_t r = (size_t)counter;
                if (rec_t) rec_t[r] = t;
                if (rec_globals) rec_globals[r] = m->g;
                orc_get_crus(m, rec_CaSS ? rec_CaSS + r * 4 * n : NULL,
                             rec_CaJSR ? rec_CaJSR + r * n : NULL, rec_LCC ? rec_LCC + r * 4 * n : NULL,
                             rec_LCCi ? rec_LCCi + r * 4 * n : NULL, rec_RyR ? rec_RyR + r * 24 * n : NULL,
                             rec_ClCh ? rec_ClCh + r * 4 * n : NULL);
            }
            ++counter;
        }
    }
    return counter;
}

void orc_cru_rates(const orc_params *p, const orc_consts *c, const int *LCC, const int *LCCi,
                   const int *RyR, const int *ClCh, const double *CaSS, double *LCC_rates,
                   double *LCCi_rates, double *RyR_rates, double *ClCh_rates,
                   double *subunit_rates) {
    orc_cru s;
    memset(&s, 0, sizeof s);
    memcpy(s.LCC, LCC, sizeof s.LCC);
    memcpy(s.LCCi, LCCi, sizeof s.LCCi);
    memcpy(s.RyR, RyR, sizeof s.RyR);
    memcpy(s.ClCh, ClCh, sizeof s.ClCh);
    memcpy(s.CaSS, CaSS, sizeof s.CaSS);
    update_rates(&s, p, c);
    memcpy(LCC_rates, s.LCC_rates, sizeof s.LCC_rates);
    memcpy(LCCi_rates, s.LCCi_rates, sizeof s.LCCi_rates);
    memcpy(RyR_rates, s.RyR_rates, sizeof s.RyR_rates);
    memcpy(ClCh_rates, s.ClCh_rates, sizeof s.ClCh_rates);
    memcpy(subunit_rates, s.subunit_rates, sizeof s.subunit_rates);
}

int orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}
