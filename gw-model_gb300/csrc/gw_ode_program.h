// gw_ode_program.h -- the global step (GW_model::euler_step, GW.tpp:237-272) as a SIMT "lane
// program" for the ODE warps of a cell's leader CTA.
//
// GB300 runs an FP64 instruction in ~34 ns per warp whether 1 or 32 lanes are active, so the
// reference's ~1400 scalar FP64 operations per step cannot be run by one thread.  The step is
// instead split into dependency phases; every op of a phase evaluates the same formula shape on
// operands picked from a slot array X[] by per-op indices, one op per lane (128 lanes = 4 warps).
// The reference's currents are rewritten as products of factors (PROD) whose linear combinations
// are formed by SUM rows; transcendental terms are evaluated in uniform LOG / SQRT / EXP / REC
// passes.  Reassociation changes results at the level of a few ulp, far inside the 1e-12 relative
// FP64 parity bound.
#pragma once

#include <cstdint>

#include "gw_internal.h"

namespace gw {

enum OdeKind : uint8_t {
    OK_NOP = 0,
    OK_LOG,   // out = log(X[a0] + X[a1]*X[a2])
    OK_SQRT,  // out = X[a0]*X[a1]*sqrt(X[a2]*X[a3])
    OK_EXP,   // out = X[a0]*exp(X[a1]*X[a2] + X[a3])
    OK_AFF,   // out = X[a0]*X[a1] + X[a2]*X[a3] + X[a4]*X[a5] + X[a6]
    OK_REC,   // out = 1 / (X[a0] + X[a1]*X[a2] + X[a3]*X[a4] + X[a5]*X[a6]*X[a7])
    OK_PROD,  // out = X[a0]*X[a1]*X[a2]*X[a3]*X[a4]*X[a5]*X[a6]
    OK_SUM,   // row of `width` lanes: out = X[a0]*X[a1] * sum over lanes and t<4 of
              //                             X[a2+3t]*X[a3+3t]*X[a4+3t]
    OK_SUMU,  // SUM row whose result is the increment of global `out`: g[out] += result (FP64
              // state) by the row's first lane, the new value to X[XS_GN + out]
};

struct OdeOp {
    uint8_t kind;
    uint8_t width;   // OK_SUM: lanes in the row (1, 2, 4 or 8); the row's first lane writes
    uint16_t out;
    uint16_t a[14];
};
static_assert(sizeof(OdeOp) == 32, "OdeOp layout");

constexpr int kOdeWarps = 4;
constexpr int kOdeLanes = 32 * kOdeWarps;
constexpr int kOdeMaxPhases = 8;
constexpr int kOdeMaxOps = 448;
constexpr int kOdeMaxAlt = 24;
constexpr int kOdeMaxSlots = 640;
constexpr int kOdeMaxConsts = kOdeConstCap;

// Fixed slots of X[].
enum OdeSlot : uint16_t {
    XS_ZERO = 0,
    XS_ONE = 1,
    XS_MONE = 2,
    XS_G = 3,                        // 36 globals (gw_globals order), read by the increments
    XS_GN = XS_G + kNumGlobals,      // the updated globals, read by the phases after the update
                                     // (copied to XS_G after the push phase)
    XS_SUMS = XS_GN + kNumGlobals,   // JLCC, ClCh, Jtr, Jxfer sums of the previous step
    XS_ISTIM = XS_SUMS + 4,
    XS_DT = XS_ISTIM + 1,
    XS_FIRST_FREE = XS_DT + 1,
};

// Per-step SSA values pushed to the CTAs (sv[]) that come from the program, by sv index.
struct alignas(16) OdeProgram {
    int n_phases;
    int phase_begin[kOdeMaxPhases + 1];  // ops [phase_begin[p], phase_begin[p+1]) of phase p (<= 128)
    int upd_phase;                       // phase of the increments and the update (OK_SUMU rows)
    int push_phase;                      // sv are pushed after this phase
    int n_slots;
    int const_begin, n_consts;           // per-cell constants occupy X[const_begin, +n_consts)
    int n_alt;
    uint16_t sv_src[kSvCount];           // X slot of each sv value (XS_ZERO if not produced)
    uint8_t wkind[kOdeMaxPhases][kOdeWarps];  // the one op kind of each warp in each phase (NOP: idle)
    uint8_t alt_idx[kOdeMaxOps];         // 255, or index of the op's variant in alt[regime-1]
    uint8_t sv_stage[kOdeMaxOps];        // 1 + the sv index an op's output is staged to for the push, or 0
    OdeOp ops[kOdeMaxOps];               // regime 0: V >= -40
    OdeOp alt[2][kOdeMaxAlt];            // regime 1: V < -40;  regime 2: V == -47.13
};
static_assert(sizeof(OdeProgram) % 16 == 0, "OdeProgram is copied in 16-byte words");

// Builds the program shared by all cells (pow_fast: all cells have Hf == Hr == 0.75, so the
// Jup powers are taken with square roots) and the per-cell constant values.
bool ode_program_build(const CellStatic &cs, bool pow_fast, OdeProgram *prog, double *consts);

// Host evaluation of one global step (FP64) in the device's operation order.
void ode_program_step_host(const OdeProgram &P, const double *consts, double *g, const double *sums,
                           double Istim, double dt, double *sv);

}  // namespace gw
