/*
 * gw_gb300.h -- C ABI of the GB300 engine for the Greenstein-Winslow (2002) canine ventricular
 * myocyte model: the per-CRU hybrid SSA and the FP64 global step, for one cell or an ensemble.
 *
 * The drop-in boundary is the reference's pybind11 module `GreensteinWinslow`
 * (lukeoloughlin/GW-model, src/pyGW.cpp:160-344, src/pyGW.hpp), which src/model.py imports as
 * build.GreensteinWinslow.  Each entry point below names the reference interface it replaces.
 *
 * Conventions
 *  - Every call returns a gw_status (GW_OK == 0).  Nothing throws across this boundary.
 *  - The caller owns every host pointer; the library owns device memory and copies in and out.
 *  - A context is used by one host thread at a time.
 *  - Arrays use the reference's layouts: CaSS [n][4] f64, CaJSR [n] f64, LCC / LCC_inactivation /
 *    ClCh [n][4] int32, RyR [n][4][6] int32 (counts of the 5 RyRs per subunit in states 1..6).
 *  - Random draws come from a counter-based stream (Philox4x32-10) keyed on
 *    (seed, cell, CRU, step, draw #), so results do not depend on launch shape or thread count.
 */
#ifndef GW_GB300_H
#define GW_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GW_ABI_VERSION 5

/* Status codes. */
typedef enum gw_status {
    GW_OK = 0,
    GW_ERR_INVALID_ARGUMENT = 1, /* bad size, pointer, option or PRNG name (Python: ValueError) */
    GW_ERR_CUDA = 2,             /* a CUDA runtime call failed */
    GW_ERR_NO_DEVICE = 3,        /* no usable sm_103 device */
    GW_ERR_EVENT_CAP = 4,        /* a CRU exceeded the per-step jump cap */
    GW_ERR_NONFINITE = 5,        /* a global state variable became NaN or Inf */
    GW_ERR_NERNST = 6,           /* non-positive concentration in a Nernst potential (the reference
                                    exits the process here, common.hpp:72-75) */
    GW_ERR_UNSUPPORTED = 7,      /* the requested launch shape does not fit this device */
    GW_ERR_OUT_OF_MEMORY = 8,
    GW_ERR_SYNC_TIMEOUT = 9      /* a bounded wait inside the engine kernel ran out (about a second
                                    for data that normally arrives within microseconds); the
                                    launch finished, its results are not valid */
} gw_status;

/* Arithmetic of the CRU state and the SSA.  The global ODE is FP64 in both. */
typedef enum gw_precision {
    GW_PRECISION_FP64 = 0, /* reference semantics, FP64 everywhere, 53-bit uniforms */
    GW_PRECISION_FP32 = 1  /* FP32 CRU state and propensities, 24-bit uniforms */
} gw_precision;

/* Model parameters: GW::Parameters<double> (src/includes/GW_utils.hpp:38-160), same members in
 * the same order, so a C++ caller may copy the reference struct member-wise. */
typedef struct gw_params {
    double T, CSA, Vcyto, VNSR, VJSR, VSS;
    int NCaRU;
    double Ko, Nao, Cao, Clo, Clcyto;
    double f, g, f1, g1, a, b, gamma0, omega, PCaL, kfClCh, kbClCh, Pto2;
    double k12, k21, k23, k32, k34, k43, k45, k54, k56, k65, k25, k52, rRyR;
    double rxfer, rtr, riss, BSRT, KBSR, BSLT, KBSL, CSQNT, KCSQN, CMDNT, KCMDN;
    double GNa, GKr, Kf, Kb, GKs;
    double GKv43, alphaa0Kv43, aaKv43, betaa0Kv43, baKv43, alphai0Kv43, aiKv43, betai0Kv43, biKv43,
        f1Kv43, f2Kv43, f3Kv43, f4Kv43, b1Kv43, b2Kv43, b3Kv43, b4Kv43;
    double PKv14, alphaa0Kv14, aaKv14, betaa0Kv14, baKv14, alphai0Kv14, aiKv14, betai0Kv14, biKv14,
        f1Kv14, f2Kv14, f3Kv14, f4Kv14, b1Kv14, b2Kv14, b3Kv14, b4Kv14;
    double Csc, GK1, KmK1, GKp, kNaCa, KmNa, KmCa, ksat, eta, INaKmax, KmNai, KmKo, IpCamax,
        KmpCa, GCab, GNab, kHTRPNp, kHTRPNm, kLTRPNp, kLTRPNm, HTRPNtot, LTRPNtot, Vmaxf, Vmaxr,
        Kmf, Kmr, Hf, Hr;
} gw_params;

/* Global (whole-cell) state: GW::GlobalState<double> (GW_utils.hpp:229-252), same order. */
typedef struct gw_globals {
    double V, Nai, Ki, Cai, CaNSR, CaLTRPN, CaHTRPN, m, h, j, xKs;
    double Kr[5];
    double Kv43[10];
    double Kv14[10];
} gw_globals;

/* Ensemble description for gw_create. */
typedef struct gw_ensemble_desc {
    int n_cells;
    const int32_t *ncru;      /* [n_cells] CRUs simulated per cell (the reference's nCRU) */
    const gw_params *params;  /* [n_cells] if params_per_cell, else [1] shared by all cells */
    int params_per_cell;
    int precision;            /* gw_precision */
    uint64_t seed;
    int device;               /* CUDA device ordinal */
    int event_cap;            /* max jumps per CRU per step; 0 -> 65536 */
    int cluster_ctas;         /* CTAs per thread-block cluster; 0 -> FP32: the smallest power of two
                                 that keeps a cell's CTAs at <= 384 CRUs, FP64: enough CTAs of at
                                 most 96 CRUs; at most 16 either way (gw_autotune measures the best
                                 choice instead) */
    int cta_crus;             /* CRU capacity of one CTA; 0 -> derived from cluster_ctas */
    int steps_per_launch;     /* global steps fused in one launch; 0 -> 1000 */
    int ode_fp32_rhs;         /* GW_PRECISION_FP32 only: 1 evaluates the global right-hand side in
                                 FP32 (state and Euler update stay FP64); 0 (default) keeps it FP64 */
    int cell_base;            /* global index of this context's cell 0: cell i draws from the streams
                                 of cell cell_base + i, so an ensemble split into contexts (one per
                                 GPU, contiguous shares) gives the results of one context holding all
                                 its cells; 0 for a whole ensemble.  cell_base + n_cells <= 2^28 */
} gw_ensemble_desc;

/* Optional recording for gw_run, mirroring record_state (pyGW.hpp:56-99): after step i of the
 * run with i % record_every == 0, record r = i / record_every (for r < max_records). */
typedef struct gw_trace {
    int64_t max_records;
    double *t;              /* [max_records] time after the step, or NULL */
    double *globals;        /* [n_cells][max_records][36] gw_globals records, or NULL */
    int cru_cell;           /* cell whose CRU arrays are recorded (below), if any */
    double *CaSS;           /* [max_records][ncru][4], or NULL */
    double *CaJSR;          /* [max_records][ncru] */
    int32_t *LCC;           /* [max_records][ncru][4] */
    int32_t *LCC_inactivation; /* [max_records][ncru][4] */
    int32_t *RyR;           /* [max_records][ncru][4][6] */
    int32_t *ClCh;          /* [max_records][ncru][4] */
    int64_t n_written;      /* out: records written */
    /* Per-record sums over each cell's CRUs, taken on the device at the record (no CRU arrays
     * leave the device): [n_cells][max_records][GW_CRU_SUMS], or NULL.  Indices GW_SUM_*. */
    double *cru_sums;
    /* The trace cell's CRU records in the reference's reduced-memory layout
     * (serialization.py:11-39): float32 Ca, int8 LCC states, bool gates and ClCh, and the RyR
     * states of each subunit as the int16 code of utils.py:8-22.  Written by the device at the
     * record step, copied as is; each NULL or [max_records][ncru][4] ([max_records][ncru] for
     * CaJSR_f32).  Not with gw_run_noalloc. */
    int8_t *LCC_i8;
    uint8_t *LCC_inactivation_u8;
    uint8_t *ClCh_u8;
    int16_t *RyR_i16;
    float *CaSS_f32;
    float *CaJSR_f32;
    /* The reference's Python current post-processing (GWSolution properties, src/model.py:771-899,
     * with the currents of :46-549) evaluated on the device at every record of every cell from the
     * record's globals and CRU sums, so no CRU array leaves the device:
     * [n_cells][max_records][GW_CURRENTS], fields GW_CUR_*, or NULL.  Not with gw_run_noalloc. */
    double *currents;
} gw_trace;

/* Last axis of gw_trace.currents: pA/pF for the currents, mM/ms for the fluxes. */
#define GW_CURRENTS 20
enum {
    GW_CUR_INA = 0, GW_CUR_INAB = 1, GW_CUR_IKR = 2, GW_CUR_IKS = 3, GW_CUR_IKV43 = 4, GW_CUR_IKV14 = 5,
    GW_CUR_ITO1 = 6, GW_CUR_IK1 = 7, GW_CUR_IKP = 8, GW_CUR_INAK = 9, GW_CUR_INACA = 10, GW_CUR_IPCA = 11,
    GW_CUR_ICAB = 12, GW_CUR_JUP = 13, GW_CUR_ICAL = 14, GW_CUR_ITO2 = 15, GW_CUR_JTR = 16, GW_CUR_JXFER = 17,
    GW_CUR_LCC_OPEN_FRACTION = 18, GW_CUR_RYR_OPEN_FRACTION = 19
};

/* Last axis of gw_trace.cru_sums.  Counts are exact; the Ca sums carry 2^-40 mM resolution. */
#define GW_CRU_SUMS 8
enum {
    GW_SUM_LCC_OPEN = 0,         /* LCC subunits in an open state (6 or 12) */
    GW_SUM_LCC_CONDUCTING = 1,   /* ... of which the voltage gate is not inactivated (= 1) */
    GW_SUM_CASS_CONDUCTING = 2,  /* sum of CaSS over the conducting subunits [mM] */
    GW_SUM_RYR_OPEN = 3,         /* RyRs in the open states 3 and 4 */
    GW_SUM_CLCH_OPEN = 4,        /* open ClCh */
    GW_SUM_CASS = 5,             /* sum of CaSS over all subunits [mM] */
    GW_SUM_CAJSR = 6,            /* sum of CaJSR over CRUs [mM] */
    GW_SUM_CRUS = 7              /* CRUs summed (= ncru) */
};

/* Run statistics. */
typedef struct gw_stats {
    uint64_t steps;          /* global steps taken by this context */
    uint64_t launches;       /* engine kernel launches */
    double kernel_ms;        /* device time of the engine kernels (CUDA events) */
    uint64_t events;         /* SSA jumps (all CRUs, all cells) */
    int cluster_ctas, cta_crus, threads_per_cta, n_clusters, ctas;
    uint64_t device_allocs;  /* cudaMalloc calls made by this library in this process so far */
} gw_stats;

typedef struct gw_ctx gw_ctx;

int gw_abi_version(void);

/* Defaults of GW::Parameters (GW_utils.hpp:40-156), GW::GlobalState (GW_utils.hpp:231-247), and
 * the Python-side GWGlobalState() (pyGW.cpp:31-76; CaLTRPN = 8.9282e-3). */
void gw_params_default(gw_params *p);
void gw_globals_default(gw_globals *g);
void gw_globals_py_default(gw_globals *g);

/* Replaces the GW_model constructor (GW.hpp:104-113) for every cell of an ensemble.  Cells start
 * from GW::GlobalState defaults, CRU state from the reference's ctor constants, JLCC = 0 and the
 * flux carry (sum Jtr, sum Jxfer) that the reference's ctor computes (GW.hpp:73-74). */
int gw_create(const gw_ensemble_desc *desc, gw_ctx **out);
int gw_destroy(gw_ctx *ctx);
/* No counterpart in the reference (it has one CPU code path).  Measures the launch shape for an
 * ensemble: for each cluster size in {16, 9, 8, 6, 4, 3, 2, 1} that fits, and for two CTA capacities each
 * (the size rule's, cta_crus = 0, and the largest that fits shared memory: fewer, fuller CTAs
 * amortise the per-step exchange between CTAs and the global step over more CRUs, which pays off for cells
 * of uneven size), builds a throwaway context from *desc (its cluster_ctas and cta_crus are
 * ignored), paces it at 1 Hz and times trial_steps global steps after a short warm-up; returns the
 * fastest cluster size, its CTA capacity (0 = size rule; best_cta_crus may be NULL) and its
 * device time per global step.  Set desc->cluster_ctas and desc->cta_crus to the results before
 * gw_create.  The contexts it builds draw their own initial states; no caller state is touched. */
int gw_autotune(const gw_ensemble_desc *desc, int trial_steps, int *best_cluster_ctas, int *best_cta_crus,
                double *best_us_per_step);

/* No counterpart in the reference.  The launch shape gw_create derives for *desc (its size rule,
 * or desc's own cluster_ctas / cta_crus where set): CTAs per cluster and CTA capacity.  Needs no
 * device.  Results depend on the shape only through each cell's CRU split, so contexts that hold
 * shares of an ensemble (cell_base) and are created with the whole ensemble's shape reproduce the
 * one-context results bit for bit. */
int gw_default_shape(const gw_ensemble_desc *desc, int *cluster_ctas, int *cta_crus);

/* Replaces GW_model::set_initial_value (GW.tpp:6-10) for one cell.  JLCC may be NULL: the
 * reference then keeps the ctor's JLCC, which is zero (GW.hpp:107-112). */
int gw_set_globals(gw_ctx *ctx, int cell, const gw_globals *g);
int gw_get_globals(gw_ctx *ctx, int cell, gw_globals *g);
int gw_set_crus(gw_ctx *ctx, int cell, const double *CaSS, const double *CaJSR,
                const int32_t *LCC, const int32_t *LCC_inactivation, const int32_t *RyR,
                const int32_t *ClCh, const double *JLCC);
int gw_get_crus(gw_ctx *ctx, int cell, double *CaSS, double *CaJSR, int32_t *LCC,
                int32_t *LCC_inactivation, int32_t *RyR, int32_t *ClCh, double *JLCC);
/* The flux sums the next step's global derivatives use (GW.tpp:188-198): sum of JLCC and of the
 * open ClCh count over CRUs and subunits (ICaL, Ito2), sum of Jtr over CRUs and of Jxfer over CRUs
 * and subunits, the last two taken at the last update_fluxes of the previous step.  gw_set_crus
 * recomputes the first two from the arrays; gw_set_flux_carry overrides all four (resume). */
int gw_set_flux_carry(gw_ctx *ctx, int cell, double sum_JLCC, double sum_ClCh, double sum_Jtr,
                      double sum_Jxfer);
int gw_get_flux_carry(gw_ctx *ctx, int cell, double *sum_JLCC, double *sum_ClCh, double *sum_Jtr,
                      double *sum_Jxfer);
/* Draws the reference's random initial CRU state (GW_utils.tpp:5-64) on the device. */
int gw_sample_initial_crus(gw_ctx *ctx, int cell);

/* Stimulus of one cell (cell < 0: all cells).  The reference evaluates a Python callable per step
 * (pyGW.hpp:114); here either a pulse train evaluated on the device at the accumulated time t
 * (Istim = amplitude when t >= start and (t - start) mod period < duration; period <= 0 means a
 * single pulse), or per-step samples Istim[i] for steps i = 0 .. n-1 of the next gw_run. */
int gw_set_stimulus_pulse(gw_ctx *ctx, int cell, double start, double period, double duration,
                          double amplitude);
int gw_set_stimulus_samples(gw_ctx *ctx, int cell, const double *Istim, int64_t n);

/* Replaces the time loop of run<PRNG> (pyGW.hpp:102-122) / GW_model::euler (GW.tpp:275-282):
 * n_steps global steps of size dt for every cell; t accumulates by t += dt. */
int gw_run(gw_ctx *ctx, double dt, int64_t n_steps, int record_every, gw_trace *trace);

/* gw_run without allocation.  No counterpart in the reference (its run<PRNG> allocates its record
 * vectors per call, pyGW.hpp:102-122).
 *
 * Same steps, records and results as gw_run, but neither device nor host memory is allocated:
 * gw_run stages the records of each launch in device buffers it cudaMallocs and cudaFrees per call
 * (cudaFree synchronizes the whole device) and converts them in host vectors.  This variant stages
 * them in one static device array of GW_NOALLOC_SCRATCH_BYTES per device, converts them to the
 * gw_trace layouts on the device and copies them straight into the caller's arrays.  It is for
 * callers that cannot allocate: a driver that steps cells from several host threads or streams,
 * where every cudaFree would stall the other streams, and processes whose device memory is held by
 * another allocator's pool (a cudaMalloc outside that pool fails although the pool has room).
 *
 * Limit: the records of one launch must fit the scratch.  Launches are shortened until they do;
 * if even 3 records do not fit, the call returns GW_ERR_INVALID_ARGUMENT with the size needed
 * (record fewer CRU fields, or use gw_run).  A record always holds the 36 globals of every cell,
 * so a globals-only trace also scales with n_cells (about 19,400 cells or more do not fit).
 * Without a trace it uses no scratch at all.
 * Set-up: every call looks the array's device address up in the current device's context
 * (cudaGetSymbolAddress; the first call on a device may load the module); make the first call on
 * each device before any stream capture begins.
 * Nothing in the scratch has to start at zero: each record slot is written by the engine before
 * it is read.  The per-cell status words are zeroed by the call itself, as gw_run does.
 * Concurrency: the scratch is shared by every context on the device.  Calls that overlap in time
 * on one device (other threads, other contexts) race on it; serialize them.  The call has
 * synchronized its stream when it returns, so consecutive calls from one thread are safe. */
#define GW_NOALLOC_SCRATCH_BYTES ((size_t)16 << 20)
int gw_run_noalloc(gw_ctx *ctx, double dt, int64_t n_steps, int record_every, gw_trace *trace);

/* Diagnostic, no counterpart in the reference: evaluates on the current device the FP64 exp and
 * log that the global step uses (table-driven, see gw_math64.cuh) for n inputs, so that their
 * error against a reference libm can be checked. */
int gw_math_check(const double *x, int64_t n, double *exp_out, double *log_out);

/* Diagnostic, no counterpart in the reference: the FP32 screen that lets the FP64 SSA lane skip
 * the FP64 rates of an iteration that is certainly the step's last, beside the FP64 iteration's
 * own decision, for n CRU states on the current device.  Per case i: chan[8i..8i+7] = LCC states,
 * flags, RyR planes 0-5 (the engine's packing, gw_get_crus' words); cass[4i..4i+3]; sv[40i..40i+39]
 * the step's SSA values (index 0 must be 0); t[i] the time reached within the step; dt[i] the step.
 * The draw is draw 0 of the stream (seed, cell 0, CRU i, step 0).  out[2i] = 1 if the screen
 * declared the iteration last, out[2i+1] = 1 if the FP64 iteration was last; jump[i] its jump
 * time when it was not (else 0).  The screen is sound if out[2i] = 1 implies out[2i+1] = 1. */
int gw_screen_check(const gw_params *p, int nCRU, int64_t n, const uint32_t *chan, const double *cass,
                    const double *sv, const double *t, const double *dt, uint64_t seed, int32_t *out,
                    double *jump);

int gw_get_time(gw_ctx *ctx, int cell, double *t, uint64_t *step);
/* Restores a cell's accumulated time and global step index (the RNG counter).  With the globals,
 * the CRU arrays including JLCC, and the flux carry, this resumes a run bit for bit; the reference
 * has no resume (its engines are seeded from std::random_device, common.hpp:19-23). */
int gw_set_time(gw_ctx *ctx, int cell, double t, uint64_t step);
int gw_get_stats(gw_ctx *ctx, gw_stats *stats);
/* Message of the last failing call on ctx (ctx may be NULL for gw_create failures). */
int gw_last_error(gw_ctx *ctx, char *msg, size_t len);

/* The global update of GW_model::euler_step (GW.tpp:237-272: currents, concentrations, gates, IKr
 * and Kv Markov chains, explicit Euler) for one cell, evaluated on the host in the engine's FP64
 * operation order (the lane program its ODE warps run).  g: the 36 globals, updated in place;
 * sums: {sum JLCC, sum ClCh, sum Jtr, sum Jxfer} of the previous step; sv (may be NULL) receives
 * the engine's 40 per-step SSA values at the updated state.  Needs no device. */
int gw_global_step_host(const gw_params *p, int nCRU, double *g, const double *sums, double Istim,
                        double dt, double *sv);

/* One-shot drop-in for the pybind11 `run` (pyGW.cpp:134-157, 341-344): simulate one cell of nCRU
 * CRUs from init_globals / init CRU arrays for num_steps steps of step_size with stimulus samples
 * Istim[num_steps] (the caller evaluates its stimulus function at t_i = sum_{k<i} step_size), and
 * record into trace every record_every steps.  prng must be one of the reference's engine names
 * (mt19937, mt19937_64, xoshiro256+, xoshiro256++, xoshiro256**, xoroshiro128+, xoroshiro128++,
 * xoroshiro128**); any other name returns GW_ERR_INVALID_ARGUMENT, as the reference raises
 * std::invalid_argument.  The engine always draws from its counter-based stream keyed on seed. */
int gw_simulate(const gw_params *p, int nCRU, double step_size, int64_t num_steps,
                const double *Istim, int record_every, const double *init_CaSS,
                const double *init_CaJSR, const int32_t *init_LCC,
                const int32_t *init_LCC_inactivation, const int32_t *init_RyR,
                const int32_t *init_ClCh, const gw_globals *init_globals, const char *prng,
                uint64_t seed, int precision, gw_trace *trace);

/* ---------------------------------------------------------------------------------------------
 * Pathwise gradients of a voltage-trace loss.  No counterpart in the reference (it has no
 * derivatives); this is the differentiation path of the model's parameter fits.
 *
 * An ensemble of cells is run forward for n_steps global steps (the same FP64 SSA lane, draws and
 * global step as gw_run with GW_PRECISION_FP64) with V sampled after every step s for which
 * (s + 1) % sample_every == 0.  gw_grad_backward takes dL/dV at the samples and returns, per cell,
 * the relative sensitivities theta_k dL/dtheta_k of the 8 parameters below, conditional on the
 * forward pass's jump trajectory: the jump times, the transitions chosen and the RyR re-splits are
 * held fixed, and the derivative of the continuous CRU updates (update_fluxes SSA.tpp:37-45,
 * update_CaSS SSA.tpp:87-99, update_CaJSR SSA.hpp:68-71, JLCC and Jrel at transitions
 * SSA.tpp:103-283) and of the global step (GW.tpp:171-212, 237-272) is taken exactly.  This
 * estimator ignores the dependence of the jump times and transition choices on the parameters.
 * Memory is bounded by checkpoints every checkpoint_every steps and a recompute of each segment.
 * ------------------------------------------------------------------------------------------- */
#define GW_GRAD_THETA 8
enum {
    GW_TH_PCAL = 0,    /* PCaL (JLCC at LCC openings) */
    GW_TH_GKR = 1,     /* GKr */
    GW_TH_GKS = 2,     /* GKs */
    GW_TH_GK1 = 3,     /* GK1 */
    GW_TH_INAKMAX = 4, /* INaKmax */
    GW_TH_VMAX = 5,    /* Vmaxf and Vmaxr scaled together (SERCA) */
    GW_TH_RRYR = 6,    /* rRyR (RyR release rate) */
    GW_TH_CSQNT = 7    /* CSQNT (JSR calsequestrin) */
};

typedef struct gw_grad_desc {
    int n_cells;
    const int32_t *ncru;      /* [n_cells] CRUs per cell */
    const gw_params *params;  /* [n_cells] if params_per_cell, else [1] */
    int params_per_cell;
    uint64_t seed;
    int device;
    double dt;                /* global step [ms] */
    int64_t n_steps;
    int checkpoint_every;     /* steps between checkpoints; 0 -> 200 */
    int sample_every;         /* V sampled after step s when (s + 1) % sample_every == 0 */
    const double *stim;       /* [n_cells][4] pulse train start, period (<= 0: single pulse),
                                 duration, amplitude, as gw_set_stimulus_pulse */
    int event_cap;            /* max jumps per CRU per step; 0 -> 65536 */
    int cell_base;            /* global index of cell 0 (random streams), as in gw_ensemble_desc */
} gw_grad_desc;

typedef struct gw_grad_stats {
    double forward_ms, backward_ms, replay_ms; /* device time of the last call of each */
    int64_t events;                            /* SSA jumps of the last forward pass */
    int64_t checkpoint_bytes, segment_bytes;   /* device memory of the checkpoints and of a segment */
} gw_grad_stats;

typedef struct gw_grad gw_grad;

int gw_grad_create(const gw_grad_desc *desc, gw_grad **out);
int gw_grad_destroy(gw_grad *g);
/* Initial state of one cell: the 36 globals and the reference's CRU arrays.  JLCC starts at zero
 * and the flux carry at the reference ctor's (GW.hpp:73-74), as gw_create leaves a cell. */
int gw_grad_set_state(gw_grad *g, int cell, const gw_globals *globals, const double *CaSS, const double *CaJSR,
                      const int32_t *LCC, const int32_t *LCC_inactivation, const int32_t *RyR, const int32_t *ClCh);
/* Runs the forward pass from the initial states; V_samples [n_cells][n_steps / sample_every] (or NULL). */
int gw_grad_forward(gw_grad *g, double *V_samples);
/* dL_dV [n_cells][n_steps / sample_every] -> sens [n_cells][GW_GRAD_THETA] relative sensitivities. */
int gw_grad_backward(gw_grad *g, const double *dL_dV, double *sens);
/* Frozen-trajectory replay: variant v re-runs cell src_cell[v] from its initial state with
 * params[v] on the jump trajectory that cell draws with its own parameters.  V_samples
 * [n_var][n_steps / sample_every]; regime_steps [n_var] (or NULL): steps begun at V >= -40 mV,
 * where the reference's h and j gate rates change form (common.hpp:176-218). */
int gw_grad_replay(gw_grad *g, int n_var, const int32_t *src_cell, const gw_params *params, double *V_samples,
                   int64_t *regime_steps);
/* Steps begun at V >= -40 mV in the last forward pass, per cell. */
int gw_grad_regime_steps(gw_grad *g, int64_t *regime_steps);
/* Globals of a cell at the end of the last forward pass. */
int gw_grad_get_globals(gw_grad *g, int cell, gw_globals *out);
int gw_grad_get_stats(gw_grad *g, gw_grad_stats *stats);
/* Message of the last failing call on g (g may be NULL for gw_grad_create failures). */
int gw_grad_last_error(gw_grad *g, char *msg, size_t len);

/* Host checks of the hand-written adjoints (no device).  gw_grad_check_global: the global
 * increment d of one step (G: 36 globals; carry: sum JLCC, sum ClCh, sum Jtr, sum Jxfer) and, for
 * a cotangent lam of G + d, the adjoints of G (identity included), of the carry sums JLCC, Jtr and
 * Jxfer, and the relative sensitivities of GKr, GKs, GK1, INaKmax and Vmax (others zero).
 * gw_grad_check_cru: one CRU step of n_sub sub-steps h[k], each followed by event ev[k] (0 none,
 * 1 subunit sub[k] starts conducting, 2 it stops, 3 its RyR open count becomes onew[k]); x =
 * CaSS[4], CaJSR, JLCC[4], open = open RyRs per subunit at the start, in = Cai, CaNSR, JLCC factors
 * JM and JE.  Returns x_out, carry_out = Jtr and the sum of Jxfer of the last sub-step, and for
 * the cotangents lam_x (of x_out) and lam_carry (of carry_out): lam_x0, lam_in (Cai, CaNSR, JM,
 * JE) and lam_par (rRyR dL/drRyR, dL/dCSQN_const). */
int gw_grad_check_global(const gw_params *p, int nCRU, const double *G, const double *carry, double Istim, double dt,
                         const double *lam, double *d, double *lam_G, double *lam_carry, double *lam_theta);
int gw_grad_check_cru(const gw_params *p, int nCRU, const double *x, const int32_t *open, const double *in, int n_sub,
                      const double *h, const int32_t *ev, const int32_t *sub, const int32_t *onew, const double *lam_x,
                      const double *lam_carry, double *x_out, double *carry_out, double *lam_x0, double *lam_in,
                      double *lam_par);

#ifdef __cplusplus
}
#endif
#endif
