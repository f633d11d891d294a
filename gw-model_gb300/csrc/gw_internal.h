// gw_internal.h -- structures shared by the host runtime (gw_capi.cpp) and the kernels.
//
// Device memory layout (one allocation per field, "planes" of length n_slots; cell c owns
// slots [slot0[c], slot0[c] + ncru[c]), padded to a multiple of 32):
//   lcc    u32  byte j = LCC state (1..12) of subunit j
//   flags  u32  bit j = LCC_inactivation of subunit j, bit 4+j = ClCh of subunit j
//   ryr    u32  x6 planes, plane k byte j = signed count of subunit j's RyRs in state k+1
//   cass   Real x4 planes (subunit j), jlcc Real x4 planes, cajsr Real, cajsr_lo f32 (FP32 only)
// 36 B of channel state per CRU plus 36 B (FP32, +4 B compensation) or 72 B (FP64) of Ca state.
#pragma once

#include <cstdint>

#include "gw_gb300.h"

namespace gw {

constexpr int kNumGlobals = 36;
constexpr int kMaxClusterCtas = 16;
constexpr int kSvCount = 40;  // per-step SSA values pushed to every CTA each step
constexpr int kSumFields = GW_CRU_SUMS;  // record-time CRU sums per cell (gw_trace.cru_sums)

// Index of per-step SSA values (sv[]) computed by a cell's ODE warp from V and pushed to the
// cell's CTAs: voltage-dependent LCC rates of update_LCC_rates (GW_utils.tpp:118-186) with the
// reference's products, inactivation rates (GW_utils.hpp:378-383) and the JLCC factors of
// GW.tpp:220-221, plus Cai/CaNSR.
enum SvIndex {
    SV_ZERO = 0,
    SV_A4 = 1, SV_A3 = 2, SV_A2 = 3, SV_A1 = 4,          // 4a, 3a, 2a, a (a = alphaLCC)
    SV_B1 = 5, SV_B2 = 6, SV_B3 = 7, SV_B4 = 8,          // b, 2b, 3b, 4b (b = betaLCC)
    SV_A4a = 9, SV_A3a = 10, SV_A2a = 11, SV_A1a = 12,   // (n*alpha)*a
    SV_B1bi = 13, SV_B2bi = 14, SV_B3bi = 15, SV_B4bi = 16,  // (n*beta)*binv
    SV_F = 17, SV_G = 18, SV_OM = 19, SV_OMB1 = 20, SV_OMB2 = 21, SV_OMB3 = 22, SV_OMB4 = 23,
    SV_F1 = 24, SV_G1 = 25,
    SV_INACT0 = 26,  // yinf/tau    (rate 0 -> 1)
    SV_INACT1 = 27,  // (1-yinf)/tau (rate 1 -> 0)
    SV_JMUL = 28, SV_JEXP = 29,
    SV_CAI = 30, SV_CANSR = 31, SV_CAI_LO = 32, SV_CANSR_LO = 33,
};

// Per-cell constant block: the parameters and the reference's Constants (GW_utils.tpp:67-116),
// computed on the host in FP64 exactly as the reference does.
constexpr int kOdeConstCap = 256;  // per-cell constants of the global-step lane program

struct CellStatic {
    gw_params p;
    double RT_F, F_RT, CRU_factor, CSA_FVcyto, VSS_Vcyto, Vcyto_VNSR, VJSR_VNSR;
    double a, gamma0, gamma0a, gamma0a2, gamma0a3, gamma0a4, binv, omega, omega_b, omega_b2,
        omega_b3, omega_b4;
    double BSR_const, BSL_const, VSS_VJSR, CSQN_const, JLCC_const, Cao_scaled, Nao3, INaCa_const,
        sigma, INaK_const, sqrtKo, PKv14_Csc, Ito2_const, IK1_const, ICaL_const, CMDN_const;
    double ode_consts[kOdeConstCap];  // constants of the lane program (gw_ode_program.h)
};

enum StimMode { STIM_NONE = 0, STIM_PULSE = 1, STIM_SAMPLES = 2 };

// Per-cell dynamic block (device resident between launches).
struct CellDyn {
    double g[kNumGlobals];  // gw_globals layout
    double t;               // accumulated time, t += dt per step
    // Flux sums over the cell's CRUs that the next global step uses (GW.tpp:188-198).
    double sum_jlcc, sum_clch, sum_jtr, sum_jxfer;
    uint64_t step;          // global step index (RNG counter)
    int stim_mode;
    int status;
    double stim_start, stim_period, stim_dur, stim_amp;
    const double *stim_samples;
    int64_t stim_n;
};

// One CTA's share of work: a contiguous CRU range of one cell.  A cell's CTAs are contiguous in
// its cluster, starting at cluster rank `first`; the first of them (the leader) runs the cell's
// global ODE.
struct CtaWork {
    int cell;
    int cru_begin;
    int cru_count;
    int rank_in_cell;
    int first;
    int n_cta_cell;
    int lead_warps;  // SSA warps of the cell's leader CTA that take CRUs (0: the leader runs only
                     // the global step, for cells spread thinly enough that it sets the step)
    int pad1;
};

struct OdeProgram;

struct KernelArgs {
    const OdeProgram *prog;
    const CtaWork *work;
    const CellStatic *cs;
    CellDyn *dyn;
    const int64_t *slot0;
    int64_t n_slots;
    uint32_t *lcc;
    uint32_t *flags;
    uint32_t *ryr;
    void *cass;
    void *jlcc;
    void *cajsr;
    float *cajsr_lo;
    double dt;
    int n_steps;
    int record_every;   // 0: no recording
    int64_t run_step0;  // run-relative index of this launch's first step
    int64_t rec_base;   // record index of the trace buffer's first slot
    int rec_cap;        // records the device trace buffers hold
    double *tr_t;       // [rec_cap]
    double *tr_glob;    // [n_cells][rec_cap][36]
    int tr_cell;        // cell whose CRU state is recorded (-1: none)
    int64_t tr_cru_stride;  // elements per record per plane (padded ncru of tr_cell)
    uint32_t *tr_lcc, *tr_flags, *tr_ryr;  // planes mode: [rec][plane][stride]; codec: tr_lcc [rec][ncru]
    void *tr_cass, *tr_cajsr;              // planes mode, Real
    int tr_mode;                           // 0: planes; 1: reduced-memory codec (AoS per CRU)
    int tr_pad;
    int64_t tr_ncru;                       // codec: CRUs of tr_cell (record stride)
    uint32_t *tr_gate, *tr_clch;           // codec: [rec][ncru] 4 bools each
    uint32_t *tr_ryrc;                     // codec: [rec][ncru][2] 4 int16 RyR codes
    float *tr_cass_f, *tr_cajsr_f;         // codec: [rec][ncru][4], [rec][ncru]
    unsigned long long *tr_sums;           // [n_cells][rec_cap][8] CRU sums (int64; Ca in 2^-40 mM)
    uint64_t seed;
    int cell_base;      // global index of cell 0: cell i draws from the streams of cell_base + i
    int event_cap;
    int n_cells;
    unsigned long long *events;
    int *status;
    int ssa_warps;      // SSA warps of a leader CTA (its kOdeWarps ODE warps follow them); the
                        // other CTAs of a cell run SSA on all ssa_warps + kOdeWarps warps
    int tile_cap;       // CRU capacity of one CTA
    int max_cta_cell;   // max CTAs of one cell (partial slot stride)
    int test_extra_tx;  // test hook, 0 in use: bytes the leader adds to the last step's expected
                        // partials (bytes no one sends), so that its bounded wait runs out
};

struct LaunchShape {
    int cluster;      // CTAs per cluster
    int threads;      // threads per CTA (SSA warps + ODE warps) * 32
    int ctas;         // grid size (multiple of cluster)
    size_t smem;      // dynamic shared memory per CTA
};

// The reference's Constants ctor (GW_utils.tpp:67-116) into a cell block (gw_capi.cpp); the
// global-step program's constants (ode_consts) are left zero.
void make_cell_static(const gw_params &p, int nCRU, CellStatic &c);
// The flux carry (sum Jtr, sum Jxfer) of the reference's ctor for n CRUs (GW.hpp:73-74).
void ctor_flux_carry(const gw_params &p, int n, double &sum_jtr, double &sum_jxfer);
// cudaMalloc of `bytes` zeroed bytes, counted in gw_stats.device_allocs (gw_capi.cpp); returns a
// cudaError_t.
int dev_alloc(void **p, size_t bytes);

// Implemented per precision in gw_kernel_fp64.cu / gw_kernel_fp32.cu.
int launch_engine_fp64(const KernelArgs &a, const LaunchShape &s, void *stream, bool ode64);
int launch_engine_fp32(const KernelArgs &a, const LaunchShape &s, void *stream, bool ode64);
size_t smem_bytes_fp64(int tile_cap, int max_cta_cell);
size_t smem_bytes_fp32(int tile_cap, int max_cta_cell);
int max_active_clusters_fp64(const LaunchShape &s, bool ode64, int *out);
int max_active_clusters_fp32(const LaunchShape &s, bool ode64, int *out);
int sample_initial_crus_dev(const KernelArgs &a, int cell, int ncru, int fp64, void *stream);
// The global step's FP64 exp and log on n device inputs (accuracy check).
int math_check_dev(const double *x, int n, double *ex, double *lg);
int screen_check_dev(const CellStatic *cs, int n, const uint32_t *chan, const double *cass, const double *sv,
                     const double *t, const double *dt, uint64_t seed, int *out, double *jump);

}  // namespace gw
