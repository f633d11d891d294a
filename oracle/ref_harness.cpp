// ref_harness.cpp -- drives the reference's own C++ (TEST INFRASTRUCTURE ONLY).
//
// Compiled by oracle/Makefile against the reference's unmodified headers
// (src/includes/{common,GW_utils,SSA,GW}.hpp and .tpp, xoshiro.hpp) and the project's Eigen-API
// shim (oracle/eigen_shim).  Output goes only to oracle/_ref/.  Two things are added around the
// reference code, nothing inside it is changed:
//
//  1. RNG injection.  InjectGen is a tag engine; urand<double, InjectGen> (common.hpp:25-29) is
//     explicitly specialised to draw from the counter-based stream defined in gw_oracle.h, keyed on
//     (seed, cell, CRU, step, draw #).  The per-CRU key is set by a specialisation of the OpenMP
//     driver GW_model<double, InjectGen>::SSA (GW.tpp:215-234), restated here with one added line
//     per CRU that opens the stream; the per-CRU work is the reference's own copy_from_CRUState,
//     SSA_single_CRU and update_CRUstate_from_temp.
//  2. Private-member access (JLCC, Jxfer, Jtr, consts, currents) through explicit instantiation of
//     member-pointer templates, to read and set the flux carry for golden records.
//
// A second entry point times the reference unmodified: GW_model<double, Xoshiro256PlusPlus>
// (the Python API's default engine, src/model.py:945) stepped by euler_step with a pulse stimulus.
#include <chrono>
#include <functional>
#include <cstdint>
#include <cstring>
#include <random>

#include "common.hpp"

extern "C" {
#include "gw_oracle.h"
}

struct InjectGen {};

namespace {
struct InjectStream {
    uint32_t key[2];
    uint32_t ctr[4];
    uint32_t buf[4];
    uint32_t k;
    int umode;
};
thread_local InjectStream t_stream;
uint64_t g_seed = 0;
uint32_t g_cell = 0;
uint64_t g_step = 0;
int g_umode = ORC_U53;
long long g_cru_draws = 0;

void open_stream(uint32_t cru) {
    InjectStream &s = t_stream;
    s.key[0] = (uint32_t)g_seed;
    s.key[1] = (uint32_t)(g_seed >> 32);
    s.ctr[0] = 0;
    s.ctr[1] = cru;
    s.ctr[2] = (uint32_t)g_step;
    s.ctr[3] = (ORC_STREAM_SSA << 28) | (g_cell & 0x0FFFFFFFu);
    s.k = 0;
    s.umode = g_umode;
}
}  // namespace

template <>
inline double urand<double, InjectGen>() {
    InjectStream &s = t_stream;
    const uint32_t half = s.k & 1u;
    if (half == 0) {
        s.ctr[0] = s.k >> 1;
        orc_philox4x32_10(s.ctr, s.key, s.buf);
    }
    ++s.k;
    const uint64_t w = ((uint64_t)s.buf[2 * half + 1] << 32) | s.buf[2 * half];
    if (s.umode == ORC_U24) {
        uint64_t m = w >> 40;
        if (m == 0) m = 1;
        return (double)m * 0x1p-24;
    }
    uint64_t m = w >> 11;
    if (m == 0) m = 1;
    return (double)m * 0x1p-53;
}

#include "GW.hpp"
#include "xoshiro.hpp"

typedef GW::GW_model<double, InjectGen> RefModel;

// Restated OpenMP driver (GW.tpp:215-234) with the per-CRU stream key added.
template <>
void GW::GW_model<double, InjectGen>::SSA(const double dt) {
    consts.alphaLCC = alphaLCC<double>(globals.V);
    consts.betaLCC = betaLCC<double>(globals.V);
    consts.yinfLCC = yinfLCC<double>(globals.V);
    consts.tauLCC = tauLCC<double>(globals.V);
    consts.JLCC_exp = square(1.0 / consts.expmVF_RT);
    consts.JLCC_multiplier = consts.JLCC_const * globals.V * consts.F_RT / (consts.JLCC_exp - 1);
#pragma omp parallel
    {
        CRUStateThread<double> temp;
#pragma omp for schedule(static)
        for (int i = 0; i < nCRU; i++) {
            open_stream((uint32_t)i);
            temp.copy_from_CRUState(CRUs, JLCC, i, parameters);
            SSA_single_CRU<double, InjectGen>(temp, globals.Cai, globals.CaNSR, dt, parameters, consts);
            update_CRUstate_from_temp(temp, i);
        }
    }
}

// ---- private-member access by explicit instantiation of member-pointer templates ----
template <typename Tag, typename Tag::type M>
struct Rob {
    friend typename Tag::type get(Tag) { return M; }
};
#define GW_ROB(name, T)                            \
    struct Tag_##name {                            \
        typedef T RefModel::*type;                 \
        friend type get(Tag_##name);               \
    };                                             \
    template struct Rob<Tag_##name, &RefModel::name>;
GW_ROB(JLCC, Array2<double>)
GW_ROB(Jxfer, Array2<double>)
GW_ROB(Jtr, Array1<double>)
GW_ROB(consts, GW::Constants<double>)
GW_ROB(currents, GW::Currents<double>)
GW_ROB(nCRU, int)

static void params_from_orc(GW::Parameters<double> &P, const orc_params *src) {
#define COPY_FIELD(t, n, d) P.n = src->n;
    ORC_PARAM_FIELDS(COPY_FIELD)
#undef COPY_FIELD
}

static void globals_to_orc(const GW::GlobalState<double> &g, orc_globals *o) {
    o->V = g.V; o->Nai = g.Nai; o->Ki = g.Ki; o->Cai = g.Cai; o->CaNSR = g.CaNSR;
    o->CaLTRPN = g.CaLTRPN; o->CaHTRPN = g.CaHTRPN; o->m = g.m; o->h = g.h; o->j = g.j;
    o->xKs = g.xKs;
    for (int i = 0; i < 5; ++i) o->Kr[i] = g.Kr[i];
    for (int i = 0; i < 10; ++i) { o->Kv14[i] = g.Kv14[i]; o->Kv43[i] = g.Kv43[i]; }
}

static void globals_from_orc(GW::GlobalState<double> &g, const orc_globals *o) {
    g.V = o->V; g.Nai = o->Nai; g.Ki = o->Ki; g.Cai = o->Cai; g.CaNSR = o->CaNSR;
    g.CaLTRPN = o->CaLTRPN; g.CaHTRPN = o->CaHTRPN; g.m = o->m; g.h = o->h; g.j = o->j;
    g.xKs = o->xKs;
    for (int i = 0; i < 5; ++i) g.Kr[i] = o->Kr[i];
    for (int i = 0; i < 10; ++i) { g.Kv14[i] = o->Kv14[i]; g.Kv43[i] = o->Kv43[i]; }
}

struct RefHandle {
    RefModel *m;
    uint64_t seed;
    uint32_t cell;
    uint64_t step;
    int umode;
};

extern "C" {

void *ref_create(const orc_params *p, int nCRU, uint64_t seed, uint32_t cell, int umode) {
    GW::Parameters<double> P;
    params_from_orc(P, p);
    RefHandle *h = new RefHandle;
    h->m = new RefModel(P, nCRU);
    h->seed = seed;
    h->cell = cell;
    h->step = 0;
    h->umode = umode;
    return h;
}

void ref_destroy(void *hv) {
    RefHandle *h = (RefHandle *)hv;
    delete h->m;
    delete h;
}

// set_initial_value (GW.tpp:6-10) with the reference's own GlobalState / CRUState types.
void ref_set_state(void *hv, const orc_globals *g, const double *CaSS, const double *CaJSR,
                   const int *LCC, const int *LCCi, const int *RyR, const int *ClCh) {
    RefHandle *h = (RefHandle *)hv;
    const int n = h->m->*get(Tag_nCRU());
    GW::GlobalState<double> G;
    globals_from_orc(G, g);
    GW::CRUState<double> C(n);
    for (int i = 0; i < n; ++i) {
        C.CaJSR(i) = CaJSR[i];
        for (int j = 0; j < 4; ++j) {
            C.CaSS(i, j) = CaSS[4 * i + j];
            C.LCC(i, j) = LCC[4 * i + j];
            C.LCC_inactivation(i, j) = LCCi[4 * i + j];
            C.ClCh(i, j) = ClCh[4 * i + j];
            for (int k = 0; k < 6; ++k) C.RyR.array(i, j, k) = RyR[24 * i + 6 * j + k];
        }
    }
    h->m->set_initial_value(G, C);
}

void ref_set_step(void *hv, uint64_t step) { ((RefHandle *)hv)->step = step; }

void ref_euler_step(void *hv, double dt, double Istim) {
    RefHandle *h = (RefHandle *)hv;
    g_seed = h->seed;
    g_cell = h->cell;
    g_step = h->step;
    g_umode = h->umode;
    h->m->Istim = Istim;
    h->m->euler_step(dt);
    ++h->step;
}

void ref_get_state(void *hv, orc_globals *g, double *CaSS, double *CaJSR, int *LCC, int *LCCi,
                   int *RyR, int *ClCh, double *JLCC, double *Jxfer, double *Jtr) {
    RefHandle *h = (RefHandle *)hv;
    RefModel &M = *h->m;
    const int n = M.*get(Tag_nCRU());
    if (g) globals_to_orc(M.globals, g);
    const Array2<double> &jl = M.*get(Tag_JLCC());
    const Array2<double> &jx = M.*get(Tag_Jxfer());
    const Array1<double> &jt = M.*get(Tag_Jtr());
    for (int i = 0; i < n; ++i) {
        if (CaJSR) CaJSR[i] = M.CRUs.CaJSR(i);
        if (Jtr) Jtr[i] = jt(i);
        for (int j = 0; j < 4; ++j) {
            if (CaSS) CaSS[4 * i + j] = M.CRUs.CaSS(i, j);
            if (LCC) LCC[4 * i + j] = M.CRUs.LCC(i, j);
            if (LCCi) LCCi[4 * i + j] = M.CRUs.LCC_inactivation(i, j);
            if (ClCh) ClCh[4 * i + j] = M.CRUs.ClCh(i, j);
            if (JLCC) JLCC[4 * i + j] = jl(i, j);
            if (Jxfer) Jxfer[4 * i + j] = jx(i, j);
            if (RyR)
                for (int k = 0; k < 6; ++k) RyR[24 * i + 6 * j + k] = M.CRUs.RyR.array(i, j, k);
        }
    }
}

// Constants (GW_utils.hpp:162-227) and Currents (GW.hpp:24-42) in declaration order.
void ref_get_consts(void *hv, orc_consts *c, orc_currents *cur) {
    RefHandle *h = (RefHandle *)hv;
    RefModel &M = *h->m;
    const GW::Constants<double> &k = M.*get(Tag_consts());
    if (c) {
        const double v[] = {k.RT_F, k.F_RT, k.CRU_factor, k.CSA_FVcyto, k.VSS_Vcyto, k.Vcyto_VNSR,
                            k.VJSR_VNSR, k.a, k.gamma0, k.gamma0a, k.gamma0a2, k.gamma0a3,
                            k.gamma0a4, k.binv, k.omega, k.omega_b, k.omega_b2, k.omega_b3,
                            k.omega_b4, k.BSR_const, k.BSL_const, k.VSS_VJSR, k.CSQN_const,
                            k.JLCC_const, k.Cao_scaled, k.Nao3, k.INaCa_const, k.sigma,
                            k.INaK_const, k.sqrtKo, k.PKv14_Csc, k.Ito2_const, k.IK1_const,
                            k.ICaL_const, k.CMDN_const, k.VF_RT, k.expmVF_RT, k.ENa, k.EK, k.ECa,
                            k.beta_cyto, k.JLCC_multiplier, k.JLCC_exp, k.alphaLCC, k.betaLCC,
                            k.yinfLCC, k.tauLCC};
        static_assert(sizeof(v) == sizeof(orc_consts), "constants layout");
        memcpy(c, v, sizeof v);
    }
    if (cur) {
        const GW::Currents<double> &I = M.*get(Tag_currents());
        const double v[] = {I.INa, I.INab, I.INaCa, I.INaK, I.IKr, I.IKs, I.Ito1, I.Ito2,
                            I.IK1, I.IKp, I.ICaL, I.ICab, I.IpCa, I.Jup, I.Jtr_tot, I.Jxfer_tot};
        static_assert(sizeof(v) == sizeof(orc_currents), "currents layout");
        memcpy(cur, v, sizeof v);
    }
}

// update_rates (SSA.tpp:48-56) of one CRU through the reference's own rate functions.
void ref_cru_rates(const orc_params *p, double V, const int *LCC, const int *LCCi, const int *RyR,
                   const int *ClCh, const double *CaSS, double *LCC_rates, double *LCCi_rates,
                   double *RyR_rates, double *ClCh_rates, double *subunit_rates) {
    GW::Parameters<double> P;
    params_from_orc(P, p);
    GW::Constants<double> C(P, 1);
    C.VF_RT = V * C.F_RT;
    C.expmVF_RT = exp(-C.VF_RT);
    C.alphaLCC = GW::alphaLCC<double>(V);
    C.betaLCC = GW::betaLCC<double>(V);
    C.yinfLCC = GW::yinfLCC<double>(V);
    C.tauLCC = GW::tauLCC<double>(V);
    GW::CRUStateThread<double> s;
    memset(&s, 0, sizeof s);
    memcpy(s.LCC, LCC, sizeof s.LCC);
    memcpy(s.LCC_inactivation, LCCi, sizeof s.LCC_inactivation);
    memcpy(s.RyR, RyR, sizeof s.RyR);
    memcpy(s.ClCh, ClCh, sizeof s.ClCh);
    memcpy(s.CaSS, CaSS, sizeof s.CaSS);
    GW::update_rates(s, P, C);
    memcpy(LCC_rates, s.LCC_rates, sizeof s.LCC_rates);
    memcpy(LCCi_rates, s.LCC_inactivation_rates, sizeof s.LCC_inactivation_rates);
    memcpy(RyR_rates, s.RyR_rates, sizeof s.RyR_rates);
    memcpy(ClCh_rates, s.ClCh_rates, sizeof s.ClCh_rates);
    memcpy(subunit_rates, s.subunit_rates, sizeof s.subunit_rates);
}

// The reference, unmodified, timed: GW_model<double, Xoshiro256PlusPlus> with random initial CRU
// state, GW::GlobalState defaults, euler_step with Istim = amp for t mod period < duration.
// Returns wall seconds for num_steps steps.
double ref_time_xoshiro(const orc_params *p, int nCRU, double dt, long long num_steps,
                        double period, double duration, double amp, int threads) {
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#endif
    GW::Parameters<double> P;
    params_from_orc(P, p);
    GW::GW_model<double, XoshiroCpp::Xoshiro256PlusPlus> model(P, nCRU);
    double t = 0.0;
    const auto t0 = std::chrono::steady_clock::now();
    for (long long i = 0; i < num_steps; ++i) {
        const double tb = t - period * (double)(long long)(t / period);
        model.Istim = (tb < duration) ? amp : 0.0;
        model.euler_step(dt);
        t += dt;
    }
    const auto t1 = std::chrono::steady_clock::now();
    return std::chrono::duration<double>(t1 - t0).count();
}

int ref_omp_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
}
