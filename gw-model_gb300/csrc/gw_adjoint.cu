// gw_adjoint.cu -- pathwise gradients of a voltage-trace loss for an ensemble of cells (gw_grad_*
// in gw_gb300.h).  No counterpart in the reference, which has no derivatives.
//
// Forward.  Per global step s, two kernels: k_ssa runs every CRU's hybrid SSA of step s (the FP64
// lane of the engine, SsaLane<double, true>, with the engine's counter-based draws keyed on (seed,
// cell, CRU, step), so the jump trajectory is the one gw_run draws); k_global sums each cell's CRU
// fluxes and takes the FP64 global step with the engine's lane program (gw_ode_program.h), as
// gw_run does.  The backward pass differentiates the reference's formulas of that step
// (gw_adjoint_math.h), which the program evaluates to a few ulp.
// The state of every CRU and cell is checkpointed every `checkpoint_every` steps.
//
// Backward, one checkpoint segment at a time from the last: the segment is recomputed from its
// checkpoint with every step's start state stored, and the CRUs whose step had a jump listed per
// step; then it is stepped in reverse:
//   k_cru_quiet   the CRUs without a jump in the step (most of them): their step is one sub-step of
//                 length dt, reversed directly from the stored start state.
//   k_cru_busy    the listed CRUs, densely packed: each re-runs its step from its stored start state
//                 with the same draws (hence the same jump times and transitions), keeps the
//                 sub-steps in blocks of kRec and walks them backwards through the adjoint of the
//                 sub-step and event arithmetic.
//   Both write per CRU its adjoint state and its adjoints of the step inputs (Cai, CaNSR, the JLCC
//   factors) and of rRyR and CSQN.
//   k_global_adj  one block per cell: sums the cell's CRU rows in a fixed order, then the adjoint
//                 of the global increment plus the CRU inputs' contributions, and the parameters'
//                 relative sensitivities.
// The SSA of a step runs with lane refill: a warp's lane whose CRU has finished its step takes the
// next CRU of the warp's range, so a CRU with many jumps does not hold 31 idle lanes.  Results do
// not depend on the order in which CRUs are processed or listed.
// Memory: (steps / checkpoint_every) checkpoints + checkpoint_every step states of every CRU.
//
// Replay (gw_grad_replay) re-runs chosen cells with other parameters on the recorded jump
// trajectory (frozen jump times and transitions): a copy of the source cell runs as in the forward
// pass and drives a variant whose continuous state follows the same sub-steps and events.  At the
// source's own parameters the replay reproduces the forward pass bit for bit, so central
// differences of replays measure exactly the derivative the adjoint computes.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "gw_adjoint_math.h"
#include "gw_engine.cuh"
#include "gw_gb300.h"
#include "gw_internal.h"
#include "gw_kernel.cuh"
#include "gw_ode_program.h"

using namespace gw;
using namespace gw::adj;

namespace {

constexpr int kBlk = 128;     // threads per block of the CRU kernels (one cell per block)
constexpr int kSsaBlocksPerSm = 3;  // k_ssa without variants: resident blocks per SM (register cap)
constexpr int kQCap = 512;    // k_ssa: CRUs per block whose first iteration runs after the block's ranges
constexpr int kRec = 16;      // sub-steps a CRU keeps per block of its reverse sweep
constexpr int kAdjIn = 6;     // per-cell CRU adjoints: Cai, CaNSR, JM, JE, rRyR (relative), CSQN_const
constexpr int kLamX = 9;      // CRU adjoint state: CaSS[4], CaJSR, JLCC[4]
using CruD = dev::Cru<double>;

struct Buf {
    void *p = nullptr;
    size_t n = 0;
    Buf() = default;
    Buf(const Buf &) = delete;
    Buf &operator=(const Buf &) = delete;
    ~Buf() {
        if (p) cudaFree(p);
    }
    int alloc(size_t bytes) {
        if (p) cudaFree(p);
        p = nullptr;
        n = bytes;
        return dev_alloc(&p, bytes);
    }
    template <typename T>
    T *as() const {
        return reinterpret_cast<T *>(p);
    }
};

// Arguments of the forward kernels for one set of cells (the ensemble, or a replay's source copies
// or variants).
struct GradArgs {
    const OdeProgram *prog;     // the global step as the engine's lane program (shared by all cells)
    const CellStatic *cs;       // [n_cells] (ode_consts: the program's per-cell constants)
    const int *blk_cell;        // [blocks] cell of each CRU block
    const int *blk_lo;          // [blocks] first CRU (within the cell) of each block
    const int *blk_hi;          // [blocks] end of the block's CRU range (within the cell)
    const int *cru_cell;        // [n_crus] cell of each CRU (backward kernels)
    const int *blk0;            // [n_cells + 1] first block of each cell
    double *part;               // [blocks][4] each block's sums of its CRUs' fluxes of the step
    const int64_t *cru0;        // [n_cells] first CRU of each cell in the CRU arrays
    const int *ncru;            // [n_cells]
    const int *rng_cell;        // [n_cells] cell index that keys the cell's random streams
    CruD *x;                    // [n_crus] CRU state
    double *out;                // [n_crus][4] the step's per-CRU sum JLCC, sum Jxfer, Jtr, open ClCh
    double *G;                  // [n_cells][36]
    double *carry;              // [n_cells][4] sum JLCC, sum ClCh, sum Jtr, sum Jxfer
    double *t;                  // [n_cells] accumulated time
    double *sv;                 // [n_cells][kSvCount] SSA values of the current step
    const double *stim;         // [n_cells][4] pulse start, period, duration, amplitude
    int *status;                // [n_cells]
    unsigned long long *events; // [n_cells] or null
    double *V;                  // [n_cells][n_samples] or null
    unsigned long long *regime; // [n_cells] steps begun at V >= -40 mV, or null
    int64_t n_samples;
    int sample_every;
    uint64_t seed;
    double dt;
    int event_cap;
    int n_cells;
    int64_t n_crus;
    // Recording of a segment's step states (null: not recording): slot = step - segment start.
    CruD *seg_x;                // [slots][n_crus]
    double *seg_G;              // [slots][n_cells][36]
    double *seg_carry;          // [slots][n_cells][4]
    double *seg_sv;             // [slots][n_cells][kSvCount]
    uint8_t *quiet;             // [slots][n_crus] 1: the CRU's step had no jump (one sub-step of dt)
    int *busy;                  // [slots][n_crus] the other CRUs of the step, in completion order
    int *busy_n;                // [slots] their count
    // Replay: the variant's continuous CRU state driven by this set's jump trajectory (null: none).
    const CellStatic *var_cs;   // [n_cells]
    double *var_x;              // [n_crus][9] CaSS[4], CaJSR, JLCC[4]
    double *var_out;            // [n_crus][4]
    double *var_part;           // [blocks][4]
    const double *var_sv;       // [n_cells][kSvCount]
};

// Adjoint arrays.
struct AdjArgs {
    double *lam_x;      // [n_crus][9]
    double *lam_G;      // [n_cells][36]
    double *lam_cy;     // [n_cells][3] adjoints of the carry sums JLCC, Jtr, Jxfer
    double *lam_th;     // [n_cells][8] relative sensitivities
    double *ai_row;     // [n_crus][kAdjIn] each CRU's adjoints of its step inputs and parameters
    double *ai_part;    // [blocks][kAdjIn] each block's sums of its CRUs' rows
    const dev::SsaConsts<double> *cc;  // [n_cells] SSA constants (k_cru_busy)
    const double *dLdV; // [n_cells][n_samples]
};

__device__ __forceinline__ double pulse_at(double t, const double *s) {
    double tb = __dsub_rn(t, s[0]);
    if (tb >= 0.0) {
        if (s[1] > 0.0) tb = __dsub_rn(tb, __dmul_rn(s[1], trunc(__ddiv_rn(tb, s[1]))));
        if (tb < s[2]) return s[3];
    }
    return 0.0;
}

// Sum of N values over the block (warp shuffles, then warp totals in order); thread 0 holds it.
template <int N>
__device__ __forceinline__ void block_sum(double (&v)[N], double *sh) {
#pragma unroll
    for (int q = 0; q < N; ++q)
        for (int off = 16; off > 0; off >>= 1) v[q] += __shfl_down_sync(0xffffffffu, v[q], off);
    const int w = (int)threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0)
        for (int q = 0; q < N; ++q) sh[w * N + q] = v[q];
    __syncthreads();
    if (threadIdx.x == 0)
        for (int q = 0; q < N; ++q) {
            double s = 0.0;
            for (int k = 0; k < kBlk / 32; ++k) s += sh[k * N + q];
            v[q] = s;
        }
}

// The cell's constant block into shared memory by the whole block (16-byte words): the serial
// global step reads ~100 of its fields, each from shared memory then instead of L2.
__device__ __forceinline__ void stage_cell(CellStatic &dst, const CellStatic &src) {
    static_assert(sizeof(CellStatic) % 16 == 0, "CellStatic is copied in 16-byte words");
    const uint4 *s = reinterpret_cast<const uint4 *>(&src);
    uint4 *d = reinterpret_cast<uint4 *>(&dst);
    for (int i = (int)threadIdx.x; i < (int)(sizeof(CellStatic) / 16); i += (int)blockDim.x) d[i] = s[i];
}

// The item of thread t when a level's items are dealt round-robin over the block's warps: each item
// takes its own code path, and a warp runs the paths of its lanes one after the other, so items
// spread over the four warps (four sub-partitions, four FP64 units) finish about 4x sooner than
// items packed into the lanes of one or two warps.
__device__ __forceinline__ int item_of(int t) { return (t & 31) * (kBlk / 32) + (t >> 5); }

__device__ __forceinline__ void open_counts(const CruD &c, int o[4]) {
#pragma unroll
    for (int j = 0; j < 4; ++j) o[j] = dev::byte_s(c.ryr[2], j) + dev::byte_s(c.ryr[3], j);
}

// The continuous effect of the transition an iteration applied (apply_event in gw_kernel.cuh),
// from the channel state before (lcc0, fl0) and after (c) it.
__device__ __forceinline__ void classify(const dev::IterInfo<double> &f, uint32_t lcc0, uint32_t fl0, const CruD &c,
                                         int &ev, int &j, int &onew) {
    ev = EV_NONE;
    j = f.aj;
    onew = 0;
    const uint32_t sh = 8u * (uint32_t)j;
    if (f.act == 1) {
        const int from = (int)((lcc0 >> sh) & 0xFFu), to = (int)((c.lcc >> sh) & 0xFFu);
        if (from >= 1 && from <= 12) {
            if ((from == 5 && to == 6) || (from == 11 && to == 12))
                ev = ((fl0 >> j) & 1u) ? EV_JLCC_SET : EV_JLCC_ZERO;
            else if (from == 6 || from == 12)
                ev = EV_JLCC_ZERO;
        }
    } else if (f.act == 2) {
        const int st = (int)((c.lcc >> sh) & 0xFFu);
        if (((c.flags >> j) & 1u) == 0u)
            ev = EV_JLCC_ZERO;
        else if (st == 6 || st == 12)
            ev = EV_JLCC_SET;
    } else if (f.act == 3) {
        ev = EV_JREL;
        onew = dev::byte_s(c.ryr[2], j) + dev::byte_s(c.ryr[3], j);
    }
}

__device__ __forceinline__ CruIn cru_in(const double *sv) {
    return CruIn{sv[SV_CAI], sv[SV_CANSR], sv[SV_JMUL], sv[SV_JEXP]};
}

// Forward SSA of step `step`: block b takes CRUs [blk_lo, blk_hi) of cell blk_cell, split evenly
// over its warps; each warp runs its range with lane refill (one SSA iteration per pass; a lane
// whose CRU finished its step takes the warp's next CRU).  CRUs whose first iteration the FP32
// screen declines (an event in the step) run after the ranges, packed into as few warps as they
// fill, so that the FP64 rate evaluations run with full lanes.
template <bool VAR>
__global__ void __launch_bounds__(kBlk, VAR ? 1 : kSsaBlocksPerSm) k_ssa(const GradArgs a, int64_t step, int slot) {
    __shared__ dev::SsaConsts<double> cc;
    __shared__ double sv[kSvCount];
    __shared__ double vsv[kSvCount];
    __shared__ double shp[(kBlk / 32) * 4];
    __shared__ float svf[kSvCount];          // float copies for the screen (SsaLane::surely_last)
    __shared__ float sk[dev::SK_COUNT];
    __shared__ int q[kQCap];                 // CRUs whose first iteration the screen declined
    __shared__ int qn;
    const int cell = a.blk_cell[blockIdx.x];
    constexpr bool var = VAR;  // the replay's variants (a.var_x and the var_* arrays set)
    if (threadIdx.x == 0) dev::load_ssa_consts<double>(cc, a.cs[cell]);
    if (threadIdx.x == 32) {
        dev::load_screen_consts(sk, a.cs[cell]);
        qn = 0;
    }
    if (threadIdx.x < kSvCount) {
        sv[threadIdx.x] = a.sv[(int64_t)cell * kSvCount + threadIdx.x];
        svf[threadIdx.x] = (float)sv[threadIdx.x];
        if (var) vsv[threadIdx.x] = a.var_sv[(int64_t)cell * kSvCount + threadIdx.x];
    }
    __syncthreads();
    const int lane = (int)threadIdx.x & 31, warp = (int)threadIdx.x >> 5;
    constexpr int nw = kBlk / 32;
    const int lo = a.blk_lo[blockIdx.x], span = a.blk_hi[blockIdx.x] - lo;
    const int end = lo + (int)((int64_t)span * (warp + 1) / nw);
    int cursor = lo + (int)((int64_t)span * warp / nw);
    const int64_t c0 = a.cru0[cell];
    const uint32_t rc = (uint32_t)a.rng_cell[cell];
    CruPar P{};
    CruIn in{};
    if (var) {
        P = cru_par(a.var_cs[cell]);
        in = cru_in(vsv);
    }
    CruD c;
    dev::SsaLane<double, true> L;
    dev::Stream rng;
    CruCont v;
    double vjtr = 0.0, vjx = 0.0;
    unsigned int ev = 0;
    int err = 0;
    // CRU mm of the cell into the lane (state, stream, Jrel; the variant's state)
    auto fetch = [&](int mm, bool first) {
        const int64_t i = c0 + mm;
        c = a.x[i];
        if (first && a.seg_x) a.seg_x[(int64_t)slot * a.n_crus + i] = c;
        rng.open(a.seed, rc, (uint32_t)mm, (uint64_t)step, 0);
        L.begin(c, cc);
        if (var) {
            // the variant follows the same sub-steps and events with its own parameters
            const double *vx = a.var_x + (int64_t)kLamX * i;
            for (int j = 0; j < 4; ++j) {
                v.c[j] = vx[j];
                v.L[j] = vx[5 + j];
            }
            v.J = vx[4];
            int o[4];
            open_counts(c, o);
            cru_begin(v, o, P);
        }
    };
    // After an iteration of CRU mm (f: what it did; lcc0, fl0: the channel state before it): the
    // variant follows it, and at the end of the step the CRU's results are written.
    auto after = [&](int mm, const dev::IterInfo<double> &f, uint32_t lcc0, uint32_t fl0, bool done) {
        if (var) {
            cru_substep(v, f.h, in, P, vjtr, vjx);
            int e, j, onew;
            classify(f, lcc0, fl0, c, e, j, onew);
            cru_event(v, e, j, onew, in, P);
        }
        if (!done) return;
        const int64_t i = c0 + mm;
        a.x[i] = c;
        double *o = a.out + 4 * i;
        o[0] = c.jlcc[0] + c.jlcc[1] + c.jlcc[2] + c.jlcc[3];
        o[1] = L.jxfer_sum;
        o[2] = L.jtr;
        o[3] = (double)__popc((c.flags >> 4) & 0xFu);
        if (var) {
            double *vx = a.var_x + (int64_t)kLamX * i;
            for (int j = 0; j < 4; ++j) {
                vx[j] = v.c[j];
                vx[5 + j] = v.L[j];
            }
            vx[4] = v.J;
            double *vo = a.var_out + 4 * i;
            vo[0] = v.L[0] + v.L[1] + v.L[2] + v.L[3];
            vo[1] = vjx;
            vo[2] = vjtr;
            vo[3] = o[3];
        }
        if (a.quiet) {
            const bool q = L.ev == 0;
            a.quiet[(int64_t)slot * a.n_crus + i] = q ? 1 : 0;
            if (!q) a.busy[(int64_t)slot * a.n_crus + atomicAdd(&a.busy_n[slot], 1)] = (int)i;
        }
        ev += (unsigned int)L.ev;
    };
    // Pass 1: the warp's CRU range, one iteration per lane and pass.  An iteration that the FP32
    // screen shows to be the step's last runs without the FP64 rates (finish).  A CRU whose first
    // iteration the screen declines is handed, untouched, to the block's queue, and its lane takes
    // the next CRU; so every pass of the range runs with full lanes.
    int m = a.status[cell] == 0 ? -1 : -2;  // CRU of this lane; -1 none yet, -2 none left
    bool fresh = false;                      // no iteration of the lane's CRU has run yet
    for (;;) {
        const unsigned need = __ballot_sync(0xffffffffu, m == -1);
        if (need) {
            const int nm = cursor + __popc(need & ((1u << lane) - 1u));
            cursor += __popc(need);
            if (m == -1) {
                if (nm < end) {
                    m = nm;
                    fetch(m, true);
                    fresh = true;
                } else {
                    m = -2;
                }
            }
        }
        if (!__any_sync(0xffffffffu, m >= 0)) break;
        if (m >= 0) {
            const uint32_t lcc0 = c.lcc, fl0 = c.flags;
            dev::IterInfo<double> f;
            bool ran = true, done = false;
            if (L.surely_last(c, cc, sk, svf, rng, a.dt)) {
                L.finish(c, cc, sv, rng, a.dt, var ? &f : nullptr);
                done = true;
            } else {
                const int qs = fresh ? atomicAdd(&qn, 1) : kQCap;
                if (qs < kQCap) {
                    q[qs] = m;
                    m = -1;
                    ran = false;
                } else {  // the queue is full, or the CRU is past its first iteration
                    done = L.iterate(c, cc, sv, nullptr, rng, a.dt, a.event_cap, err, var ? &f : nullptr);
                }
            }
            fresh = false;
            if (ran) {
                after(m, f, lcc0, fl0, done);
                if (done) m = -1;
            }
        }
    }
    // Pass 2: the queued CRUs (those with an event, and the few the screen's margins declined), on
    // as few warps as they fill.  Their first iteration runs in FP64; later ones are screened, and
    // a declined one waits (pend) until kDefer lanes of the warp wait or the warp has no queued
    // CRUs left, then they run the FP64 iteration together.
    __syncthreads();
    const int nq = min(qn, kQCap);
    if constexpr (!VAR) {
        // Four lanes per queued CRU (SsaLane::iterate_group: one subunit's rates per lane), eight
        // CRUs per warp at a time: the queue is the tail of the block's step, so its FP64
        // iterations are taken at a third of their single-lane latency.
        const int j = lane & 3, base = lane & ~3;
        const int nwu = min(nw, (nq + 7) >> 3);
        if (warp < nwu) {
            int qc = (int)((int64_t)nq * warp / nwu);
            const int qe = (int)((int64_t)nq * (warp + 1) / nwu);
            m = -1;
            bool first = false;  // the CRU's first iteration (declined by the screen in pass 1)
            for (;;) {
                const unsigned need = __ballot_sync(0xffffffffu, m == -1 && j == 0);
                if (need) {
                    const int nm = qc + __popc(need & ((1u << base) - 1u));
                    qc += __popc(need);
                    if (m == -1) {
                        if (nm < qe) {
                            m = q[nm];
                            fetch(m, false);
                            first = true;
                        } else {
                            m = -2;
                        }
                    }
                }
                if (!__any_sync(0xffffffffu, m >= 0)) break;
                if (m >= 0) {
                    bool done;
                    if (!first && L.surely_last(c, cc, sk, svf, rng, a.dt)) {
                        L.finish(c, cc, sv, rng, a.dt);
                        done = true;
                    } else {
                        done = L.iterate_group(c, cc, sv, rng, a.dt, a.event_cap, err);
                    }
                    first = false;
                    if (done) {
                        if (j == 0) after(m, dev::IterInfo<double>{}, 0u, 0u, true);
                        m = -1;
                    }
                }
            }
        }
    }
    if constexpr (VAR) {
        const int nwu = min(nw, (nq + 31) >> 5);
        if (warp < nwu) {
            int qc = (int)((int64_t)nq * warp / nwu);
            const int qe = (int)((int64_t)nq * (warp + 1) / nwu);
            m = -1;
            bool pend = false;  // the lane's next iteration needs the FP64 rates
            for (;;) {
                const unsigned need = __ballot_sync(0xffffffffu, m == -1);
                if (need) {
                    const int nm = qc + __popc(need & ((1u << lane) - 1u));
                    qc += __popc(need);
                    if (m == -1) {
                        if (nm < qe) {
                            m = q[nm];
                            fetch(m, false);
                            pend = true;
                        } else {
                            m = -2;
                        }
                    }
                }
                if (!__any_sync(0xffffffffu, m >= 0)) break;
                const uint32_t lcc0 = c.lcc, fl0 = c.flags;
                dev::IterInfo<double> f;
                bool ran = false, done = false;
                if (m >= 0 && !pend) {
                    if (L.surely_last(c, cc, sk, svf, rng, a.dt)) {
                        L.finish(c, cc, sv, rng, a.dt, var ? &f : nullptr);
                        ran = done = true;
                    } else {
                        pend = true;
                    }
                }
                const unsigned pm = __ballot_sync(0xffffffffu, pend);
                if (pm && (qc >= qe || __popc(pm) >= dev::kDefer) && pend) {
                    done = L.iterate(c, cc, sv, nullptr, rng, a.dt, a.event_cap, err, var ? &f : nullptr);
                    ran = true;
                    pend = false;
                }
                if (ran) {
                    after(m, f, lcc0, fl0, done);
                    if (done) m = -1;
                }
            }
        }
    }
    const unsigned int wev = __reduce_add_sync(0xffffffffu, ev);
    if (a.events && lane == 0 && wev) atomicAdd(&a.events[cell], (unsigned long long)wev);
    if (err) atomicExch(&a.status[cell], (int)GW_ERR_EVENT_CAP);
    // The block's flux sums over its CRU range, in a fixed order (the lanes took the CRUs in the
    // order they finished, so per-lane sums would not be reproducible).
    __syncthreads();
    for (int w = 0; w < (var ? 2 : 1); ++w) {
        const double *rows = (w ? a.var_out : a.out) + 4 * c0;
        double s4[4] = {0.0, 0.0, 0.0, 0.0};
        for (int m = lo + (int)threadIdx.x; m < lo + span; m += kBlk)
            for (int q = 0; q < 4; ++q) s4[q] += rows[4 * (int64_t)m + q];
        block_sum<4>(s4, shp);
        if (threadIdx.x == 0)
            for (int q = 0; q < 4; ++q) (w ? a.var_part : a.part)[4 * (int64_t)blockIdx.x + q] = s4[q];
        __syncthreads();
    }
}

// Shared-memory layout of k_global: the engine's global-step data (OdeShared, the lane program, its
// slot array, the exp/log tables, the staging row of the SSA values), as ode_phase addresses them.
struct GlobalLayout {
    uint32_t ode, prog, x, math, stage, total;
};
__host__ __device__ inline GlobalLayout global_layout() {
    auto a16 = [](size_t n) { return (uint32_t)((n + 15) & ~(size_t)15); };
    GlobalLayout L;
    uint32_t o = 0;
    L.ode = o;
    o += a16(sizeof(dev::OdeShared));
    L.prog = o;
    o += a16(sizeof(OdeProgram));
    L.x = o;
    o += a16(kOdeMaxSlots * sizeof(double));
    L.math = o;
    o += a16(sizeof(math64::Tables));
    L.stage = o;
    o += a16(kSvCount * sizeof(double));
    L.total = o;
    return L;
}

// The cell's flux sums of the step (its blocks' partial sums, in block order) and its global step,
// one block of the engine's kOdeLanes threads per cell running the engine's lane program
// (gw_ode_program.h): every warp holds one op kind per phase, so a phase costs about one op.  The
// program's transcendental phases of the step's state run first (the engine keeps them from the
// previous step; a block here starts from the recorded globals), then the increments with the
// update, then the phases up to the SSA values of the new state, which are staged as the engine
// pushes them.
__global__ void __launch_bounds__(kOdeLanes) k_global(const GradArgs a, int64_t step, int slot, int use_var) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ double sums[4];
    const GlobalLayout L = global_layout();
    dev::OdeShared &os = *reinterpret_cast<dev::OdeShared *>(smem + L.ode);
    OdeProgram &P = *reinterpret_cast<OdeProgram *>(smem + L.prog);
    double *X = reinterpret_cast<double *>(smem + L.x);
    double *stage = reinterpret_cast<double *>(smem + L.stage);
    const dev::OdeOffsets off{L.prog, L.x, L.ode, L.math, L.stage};
    const int cell = blockIdx.x;
    if (a.status[cell] != 0) return;  // the same for the whole block
    const int t = (int)threadIdx.x;
    const CellStatic &C = use_var ? a.var_cs[cell] : a.cs[cell];
    double *g = a.G + (int64_t)kNumGlobals * cell;
    double *cy = a.carry + 4 * (int64_t)cell;
    double *svo = (use_var ? const_cast<double *>(a.var_sv) : a.sv) + (int64_t)kSvCount * cell;
    {
        const int4 *src = reinterpret_cast<const int4 *>(a.prog);
        int4 *dst = reinterpret_cast<int4 *>(&P);
        for (int i = t; i < (int)(sizeof(OdeProgram) / 16); i += kOdeLanes) dst[i] = src[i];
    }
    math64::load_tables(*reinterpret_cast<math64::Tables *>(smem + L.math), t, kOdeLanes);
    for (int i = t; i < kOdeMaxSlots; i += kOdeLanes) X[i] = 0.0;
    if (t < 4) {
        const double *pp = use_var ? a.var_part : a.part;
        double v = 0.0;
        for (int b = a.blk0[cell]; b < a.blk0[cell + 1]; ++b) v += pp[4 * (int64_t)b + t];
        sums[t] = v;
    }
    // the step's record (before anything of it is overwritten)
    if (a.seg_G) {
        const int64_t r = (int64_t)slot * a.n_cells + cell;
        if (t < kNumGlobals) a.seg_G[r * kNumGlobals + t] = g[t];
        if (t < 4) a.seg_carry[r * 4 + t] = cy[t];
        if (t < kSvCount) a.seg_sv[r * kSvCount + t] = svo[t];
    }
    __syncthreads();
    if (t == 0) {
        X[XS_ONE] = 1.0;
        X[XS_MONE] = -1.0;
        X[XS_DT] = a.dt;
        X[XS_ISTIM] = pulse_at(a.t[cell], a.stim + 4 * (int64_t)cell);
        for (int q = 0; q < 4; ++q) X[XS_SUMS + q] = cy[q];
        os.status = 0;
        if (a.regime && g[0] >= -40.0) a.regime[cell] += 1ull;
    }
    if (t < kNumGlobals) {
        os.g[t] = g[t];
        X[XS_G + t] = X[XS_GN + t] = g[t];
    }
    for (int i = t; i < kOdeConstCap; i += kOdeLanes) X[XS_FIRST_FREE + i] = C.ode_consts[i];
    __syncthreads();
    const int reg = dev::v_regime(os.g[0]);
    for (int q = P.upd_phase + 1; q < P.n_phases; ++q) {
        dev::ode_phase<double, double>(off, q, reg, t);
        __syncthreads();
    }
    const bool nernst = dev::not_positive(os.g[1]) || dev::not_positive(os.g[2]);
    for (int q = 0; q <= P.upd_phase; ++q) {
        dev::ode_phase<double, double>(off, q, reg, t);
        __syncthreads();
    }
    // the SSA values of the new state: the constant ones from their slots, the others from the
    // program's phases up to the push, Cai and CaNSR from the new globals
    if (t < kSvCount && t != SV_CAI && t != SV_CANSR && t != SV_CAI_LO && t != SV_CANSR_LO &&
        P.sv_src[t] < XS_FIRST_FREE + kOdeMaxConsts)
        stage[t] = X[P.sv_src[t]];
    const int reg2 = dev::v_regime(os.g[0]);
    for (int q = P.upd_phase + 1; q <= P.push_phase; ++q) {
        dev::ode_phase<double, double>(off, q, reg2, t);
        __syncthreads();
    }
    if (t == 0) {
        dev::stage_pair(stage, SV_CAI, SV_CAI_LO, os.g[3]);
        dev::stage_pair(stage, SV_CANSR, SV_CANSR_LO, os.g[4]);
        if (nernst) {
            a.status[cell] = GW_ERR_NERNST;
        } else if (os.status != 0) {
            a.status[cell] = os.status;
        } else {
            // carry order {JLCC, ClCh, Jtr, Jxfer} from the per-CRU {JLCC, Jxfer, Jtr, ClCh}
            cy[0] = sums[0];
            cy[1] = sums[3];
            cy[2] = sums[2];
            cy[3] = sums[1];
            a.t[cell] += a.dt;
            if (a.V && (step + 1) % a.sample_every == 0) {
                const int64_t si = (step + 1) / a.sample_every - 1;
                if (si < a.n_samples) a.V[(int64_t)cell * a.n_samples + si] = os.g[0];
            }
        }
    }
    __syncthreads();
    if (nernst || os.status != 0) return;
    if (t < kNumGlobals) g[t] = os.g[t];
    if (t < kSvCount) svo[t] = stage[t];
}

// The adjoint state of CRU i after its step (its lam_x row, and the carry adjoints: the step's
// sum of JLCC is the sum of the final JLCC).
__device__ __forceinline__ CruCont lam_after(const double *lx, const double *lc) {
    CruCont la;
    for (int j = 0; j < 4; ++j) {
        la.c[j] = lx[j];
        la.L[j] = lx[5 + j] + lc[0];
        la.rel[j] = 0.0;
    }
    la.J = lx[4];
    return la;
}

__device__ __forceinline__ CruCont cont_of(const CruD &x) {
    CruCont s;
    for (int j = 0; j < 4; ++j) {
        s.c[j] = x.cass[j];
        s.L[j] = x.jlcc[j];
        s.rel[j] = 0.0;
    }
    s.J = x.cajsr;
    return s;
}

__device__ __forceinline__ void store_adj(const CruCont &la, const CruAdjIn &ai, double *lx, double *row) {
    for (int j = 0; j < 4; ++j) {
        lx[j] = la.c[j];
        lx[5 + j] = la.L[j];
    }
    lx[4] = la.J;
    row[0] = ai.Cai;
    row[1] = ai.CaNSR;
    row[2] = ai.JM;
    row[3] = ai.JE;
    row[4] = ai.rRyR_rel;
    row[5] = ai.CSQN;
}

// Reverse of step `slot` for the CRUs whose step had no jump: one sub-step of length dt (the
// iteration's h = dt - 0) and no transition.  Block b takes the CRU range of the forward block
// tables; after its CRUs it sums all its range's rows (the listed CRUs' rows come from k_cru_busy,
// launched before it) in a fixed order into ai_part[b].
__global__ void __launch_bounds__(kBlk) k_cru_quiet(const GradArgs a, const AdjArgs b, int slot) {
    __shared__ double shp[(kBlk / 32) * kAdjIn];
    const int cell = a.blk_cell[blockIdx.x];
    const int lo = a.blk_lo[blockIdx.x], hi = a.blk_hi[blockIdx.x];
    const int64_t c0 = a.cru0[cell];
    const CruPar P = cru_par(a.cs[cell]);
    const CruIn in = cru_in(a.seg_sv + ((int64_t)slot * a.n_cells + cell) * kSvCount);
    const double *lc = b.lam_cy + 3 * (int64_t)cell;
    for (int m = lo + (int)threadIdx.x; m < hi; m += kBlk) {
        const int64_t i = c0 + m;
        if (!a.quiet[(int64_t)slot * a.n_crus + i]) continue;
        const CruD x0 = a.seg_x[(int64_t)slot * a.n_crus + i];
        double *lx = b.lam_x + (int64_t)kLamX * i;
        CruCont la = lam_after(lx, lc);
        CruAdjIn ai{0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        int o[4];
        open_counts(x0, o);
        CruCont s0 = cont_of(x0);
        cru_begin(s0, o, P);
        cru_substep_adj(s0, a.dt, in, P, lc[1], lc[2], la, ai);
        cru_begin_adj(s0, o, P, la, ai);
        store_adj(la, ai, lx, b.ai_row + (int64_t)kAdjIn * i);
    }
    __syncthreads();
    double s6[kAdjIn] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int m = lo + (int)threadIdx.x; m < hi; m += kBlk)
        for (int q = 0; q < kAdjIn; ++q) s6[q] += b.ai_row[(int64_t)kAdjIn * (c0 + m) + q];
    block_sum<kAdjIn>(s6, shp);
    if (threadIdx.x == 0)
        for (int q = 0; q < kAdjIn; ++q) b.ai_part[(int64_t)kAdjIn * blockIdx.x + q] = s6[q];
}

// One recorded sub-step of a CRU's step: the state at its start and what ended it.
struct Rec {
    CruCont s;
    double h;
    int ev, j, onew;
};

// Re-runs a CRU's step from x0 and keeps iterations [lo, hi) in rec[k % kRec]; stops after hi
// iterations or at the end of the step.  Returns the iterations run.
__device__ int run_rec(const CruD &x0, const dev::SsaConsts<double> &cc, const double *sv, uint64_t seed,
                       uint32_t rcell, uint32_t m, uint64_t step, double dt, int cap, int lo, int hi, Rec *rec) {
    CruD c = x0;
    dev::Stream rng;
    rng.open(seed, rcell, m, step, 0);
    dev::SsaLane<double, true> L;
    L.begin(c, cc);
    int k = 0, err = 0;
    for (;;) {
        CruCont s;
        const bool keep = k >= lo && k < hi;
        if (keep) {
            for (int j = 0; j < 4; ++j) {
                s.c[j] = c.cass[j];
                s.L[j] = c.jlcc[j];
                s.rel[j] = L.jrel[j];
            }
            s.J = c.cajsr;
        }
        const uint32_t lcc0 = c.lcc, fl0 = c.flags;
        dev::IterInfo<double> f;
        const bool done = L.iterate(c, cc, sv, nullptr, rng, dt, cap, err, &f);
        if (keep) {
            Rec &r = rec[k % kRec];
            r.s = s;
            r.h = f.h;
            classify(f, lcc0, fl0, c, r.ev, r.j, r.onew);
        }
        ++k;
        if (done || k >= hi) break;
    }
    return k;
}

// Reverse of step `step` for the CRUs the recompute listed (their step had jumps), one thread per
// listed CRU: the step is re-run from its stored start state (same draws, same trajectory) to
// recover the sub-steps, kRec at a time from the last block, and each block is reversed.
__global__ void __launch_bounds__(kBlk) k_cru_busy(const GradArgs a, const AdjArgs b, int64_t step, int slot) {
    const int nb = a.busy_n[slot];
    for (int k = (int)(blockIdx.x * kBlk + threadIdx.x); k < nb; k += (int)(gridDim.x * kBlk)) {
        const int64_t i = a.busy[(int64_t)slot * a.n_crus + k];
        const int cell = a.cru_cell[i];
        const uint32_t m = (uint32_t)(i - a.cru0[cell]);
        const dev::SsaConsts<double> &cc = b.cc[cell];
        const double *sv = a.seg_sv + ((int64_t)slot * a.n_cells + cell) * kSvCount;
        const CruD x0 = a.seg_x[(int64_t)slot * a.n_crus + i];
        const CruPar P = cru_par(a.cs[cell]);
        const CruIn in = cru_in(sv);
        const double *lc = b.lam_cy + 3 * (int64_t)cell;
        double *lx = b.lam_x + (int64_t)kLamX * i;
        CruCont la = lam_after(lx, lc);
        CruAdjIn ai{0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        Rec rec[kRec];
        const uint32_t rc = (uint32_t)a.rng_cell[cell];
        const int n = run_rec(x0, cc, sv, a.seed, rc, m, (uint64_t)step, a.dt, a.event_cap, 0, 1 << 30, rec);
        for (int blk = (n - 1) / kRec; blk >= 0; --blk) {
            const int lo = blk * kRec, hi = min(n, lo + kRec);
            if (blk != (n - 1) / kRec) run_rec(x0, cc, sv, a.seed, rc, m, (uint64_t)step, a.dt, a.event_cap, lo, hi, rec);
            for (int q = hi - 1; q >= lo; --q) {
                const Rec &r = rec[q % kRec];
                CruCont s1 = r.s;
                double jt, jx;
                cru_substep(s1, r.h, in, P, jt, jx);
                cru_event_adj(s1, r.ev, r.j, r.onew, in, P, la, ai);
                const bool last = q == n - 1;
                cru_substep_adj(r.s, r.h, in, P, last ? lc[1] : 0.0, last ? lc[2] : 0.0, la, ai);
            }
        }
        int o[4];
        open_counts(x0, o);
        cru_begin_adj(cont_of(x0), o, P, la, ai);
        store_adj(la, ai, lx, b.ai_row + (int64_t)kAdjIn * i);
    }
}

// Reverse of the global step `step` (one block per cell): the cell's block sums of the CRU rows, the
// increment's transcendental terms one per thread, the kAdjParts parts of the increment's adjoint
// one per thread into rows summed in a fixed order, then the CRU inputs' contributions.
constexpr int kAdjOut = kNumGlobals + 3 + kTheta;  // lam_g, lam_cy, lam_th of one part
__global__ void __launch_bounds__(kBlk) k_global_adj(const GradArgs a, const AdjArgs b, int64_t step, int slot) {
    __shared__ double T[kNT];
    __shared__ double sai[kAdjIn];
    __shared__ double lam[kNumGlobals];
    __shared__ double rows[kAdjParts][kAdjOut];
    __shared__ double tot[kAdjOut];
    __shared__ __align__(16) CellStatic C;
    const int cell = blockIdx.x;
    const int t = (int)threadIdx.x;
    stage_cell(C, a.cs[cell]);
    if (t < kAdjIn) {
        double v = 0.0;
        for (int k = a.blk0[cell]; k < a.blk0[cell + 1]; ++k) v += b.ai_part[(int64_t)kAdjIn * k + t];
        sai[t] = v;
    }
    const int64_t r = (int64_t)slot * a.n_cells + cell;
    const double *g = a.seg_G + r * kNumGlobals;
    const double *cyv = a.seg_carry + r * 4;
    const Carry cy{cyv[0], cyv[1], cyv[2], cyv[3]};
    double *lgp = b.lam_G + (int64_t)kNumGlobals * cell;
    if (t < kNumGlobals) {
        double v = lgp[t];
        if (t == 0 && (step + 1) % a.sample_every == 0) {
            const int64_t si = (step + 1) / a.sample_every - 1;
            if (si < a.n_samples) v += b.dLdV[(int64_t)cell * a.n_samples + si];
        }
        lam[t] = v;
    }
    __syncthreads();
    const int it = item_of(t);
    if (it < kNT) T[it] = glob_term(C, g, it);
    __syncthreads();
    if (it < kAdjParts) {
        double *row = rows[it];
        for (int k = 0; k < kAdjOut; ++k) row[k] = 0.0;
        glob_increment_adj(C, g, cy, a.dt, T, lam, it, row, row + kNumGlobals, row + kNumGlobals + 3);
    }
    __syncthreads();
    if (t < kAdjOut) {
        double v = 0.0;
        for (int q = 0; q < kAdjParts; ++q) v += rows[q][t];
        tot[t] = v;
    }
    __syncthreads();
    if (t != 0) return;
    const double *sv = a.seg_sv + r * kSvCount;
    double lg[kNumGlobals];
    for (int k = 0; k < kNumGlobals; ++k) lg[k] = tot[k];
    double *th = b.lam_th + (int64_t)kTheta * cell;
    double lth[kTheta];
    for (int k = 0; k < kTheta; ++k) lth[k] = th[k] + tot[kNumGlobals + 3 + k];
    // the CRUs' step inputs: Cai, CaNSR and the JLCC factors of V
    lg[3] += sai[0];
    lg[4] += sai[1];
    double dJM, dJE;
    jlcc_factor_derivs(C, g[0], sv[SV_JEXP], dJM, dJE);
    lg[0] += sai[2] * dJM + sai[3] * dJE;
    lth[TH_PCAL] += sai[2] * sv[SV_JMUL];
    lth[TH_RRYR] += sai[4];
    lth[TH_CSQNT] += sai[5] * C.CSQN_const;
    for (int k = 0; k < kNumGlobals; ++k) lgp[k] = lg[k];
    for (int k = 0; k < 3; ++k) b.lam_cy[3 * (int64_t)cell + k] = tot[kNumGlobals + k];
    for (int k = 0; k < kTheta; ++k) th[k] = lth[k];
}

// SSA constants of every cell, for the kernels whose threads mix cells.
__global__ void k_init_consts(const CellStatic *cs, dev::SsaConsts<double> *cc, int n_cells) {
    const int c = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (c < n_cells) dev::load_ssa_consts<double>(cc[c], cs[c]);
}

int fail_to(std::string &err, int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    err = buf;
    return code;
}

thread_local std::string g_grad_create_error;

// Host CRU record of the reference's arrays for one CRU (JLCC zero, as the reference's ctor).
int pack_cru(const double *CaSS, const double *CaJSR, const int32_t *LCC, const int32_t *LCCi, const int32_t *RyR,
             const int32_t *ClCh, int i, CruD &c, double &clch) {
    std::memset(&c, 0, sizeof c);
    for (int j = 0; j < 4; ++j) {
        const int s = LCC[4 * i + j], li = LCCi[4 * i + j], ch = ClCh[4 * i + j];
        if (s < 1 || s > 12 || (li != 0 && li != 1) || (ch != 0 && ch != 1)) return 1;
        c.lcc |= (uint32_t)(s & 0xFF) << (8 * j);
        c.flags |= (uint32_t)li << j;
        c.flags |= (uint32_t)ch << (4 + j);
        clch += ch;
        for (int k = 0; k < 6; ++k) {
            const int v = RyR[24 * i + 6 * j + k];
            if (v < -128 || v > 127) return 1;
            c.ryr[k] |= (uint32_t)(v & 0xFF) << (8 * j);
        }
        c.cass[j] = CaSS[4 * i + j];
        c.jlcc[j] = 0.0;
    }
    c.cajsr = CaJSR[i];
    return 0;
}

// Blocks of k_ssa for cells of ncru[] CRUs: a cell gets blocks in proportion to its CRUs, rounded
// down so that all of them fit the device's `slots` resident blocks in one wave (at least one, at
// most one per 32 CRUs); block r of bpc takes CRUs [ncru r / bpc, ncru (r + 1) / bpc).
void plan_blocks(const std::vector<int> &ncru, int slots, std::vector<int> &bc, std::vector<int> &bl,
                 std::vector<int> &bh, std::vector<int> &b0) {
    int64_t total = 0;
    for (int n : ncru) total += n;
    bc.clear();
    bl.clear();
    bh.clear();
    b0.assign(ncru.size() + 1, 0);
    for (size_t c = 0; c < ncru.size(); ++c) {
        b0[c] = (int)bc.size();
        const int64_t n = ncru[c];
        int64_t bpc = (int64_t)((double)slots * (double)n / (double)total);
        bpc = std::max<int64_t>(1, std::min<int64_t>(bpc, (n + 31) / 32));
        for (int64_t r = 0; r < bpc; ++r) {
            bc.push_back((int)c);
            bl.push_back((int)(n * r / bpc));
            bh.push_back((int)(n * (r + 1) / bpc));
        }
    }
    b0[ncru.size()] = (int)bc.size();
}

}  // namespace

struct gw_grad {
    int device = 0;
    int n_cells = 0;
    int64_t n_crus = 0;
    int n_blocks = 0;
    int sm_count = 1, slots = 1;  // SMs, and resident k_ssa blocks on the device
    std::vector<int> ncru, blk_cell, blk_lo, blk_hi, blk0, cru_cell;
    std::vector<int64_t> cru0;
    std::vector<CellStatic> cs;
    std::vector<double> stim;
    double dt = 0.0;
    int64_t n_steps = 0, n_samples = 0, n_ck = 0;
    int ck_every = 200, sample_every = 1, event_cap = 65536, cell_base = 0;
    uint64_t seed = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::string err;
    std::vector<char> have_state;
    OdeProgram prog{};
    bool forwarded = false;
    gw_grad_stats stats{};
    std::vector<double> G_final;
    // tables
    Buf d_cs, d_prog, d_blk_cell, d_blk_lo, d_blk_hi, d_blk0, d_cru_cell, d_cru0, d_ncru, d_rng_cell, d_stim, d_cc;
    // initial state
    Buf x_init, G_init, carry_init, sv_init;
    // state
    Buf x, out, part, G, carry, t, sv, status, events, V, regime;
    // checkpoints and segment
    Buf ck_x, ck_G, ck_carry, ck_t, ck_sv;
    Buf seg_x, seg_G, seg_carry, seg_sv, quiet, busy, busy_n;
    // adjoint
    Buf lam_x, lam_G, lam_cy, lam_th, ai_row, ai_part, dLdV;

    ~gw_grad() {
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (stream) cudaStreamDestroy(stream);
    }
    int cuda(cudaError_t e, const char *what) {
        if (e == cudaSuccess) return GW_OK;
        cudaGetLastError();
        return fail_to(err, e == cudaErrorMemoryAllocation ? GW_ERR_OUT_OF_MEMORY : GW_ERR_CUDA, "%s: %s", what,
                       cudaGetErrorString(e));
    }
    int alloc(Buf &b, size_t bytes, const char *what) {
        const int e = b.alloc(bytes);
        return cuda((cudaError_t)e, what);
    }
    GradArgs args() const {
        GradArgs a{};
        a.prog = d_prog.as<OdeProgram>();
        a.cs = d_cs.as<CellStatic>();
        a.blk_cell = d_blk_cell.as<int>();
        a.blk_lo = d_blk_lo.as<int>();
        a.blk_hi = d_blk_hi.as<int>();
        a.cru_cell = d_cru_cell.as<int>();
        a.blk0 = d_blk0.as<int>();
        a.part = part.as<double>();
        a.cru0 = d_cru0.as<int64_t>();
        a.ncru = d_ncru.as<int>();
        a.rng_cell = d_rng_cell.as<int>();
        a.x = x.as<CruD>();
        a.out = out.as<double>();
        a.G = G.as<double>();
        a.carry = carry.as<double>();
        a.t = t.as<double>();
        a.sv = sv.as<double>();
        a.stim = d_stim.as<double>();
        a.status = status.as<int>();
        a.events = events.as<unsigned long long>();
        a.V = V.as<double>();
        a.regime = regime.as<unsigned long long>();
        a.n_samples = n_samples;
        a.sample_every = sample_every;
        a.seed = seed;
        a.dt = dt;
        a.event_cap = event_cap;
        a.n_cells = n_cells;
        a.n_crus = n_crus;
        return a;
    }
    AdjArgs adj_args() const {
        AdjArgs b{};
        b.lam_x = lam_x.as<double>();
        b.lam_G = lam_G.as<double>();
        b.lam_cy = lam_cy.as<double>();
        b.lam_th = lam_th.as<double>();
        b.ai_row = ai_row.as<double>();
        b.ai_part = ai_part.as<double>();
        b.cc = d_cc.as<dev::SsaConsts<double>>();
        b.dLdV = dLdV.as<double>();
        return b;
    }
    // Restores the state of step s0 = k * ck_every from checkpoint k (k = -1: the initial state).
    int restore(int64_t k) {
        const size_t xb = sizeof(CruD) * n_crus, gb = sizeof(double) * kNumGlobals * n_cells;
        const size_t cb = sizeof(double) * 4 * n_cells, tb = sizeof(double) * n_cells;
        const size_t sb = sizeof(double) * kSvCount * n_cells;
        int rc;
        if (k < 0) {
            if ((rc = cuda(cudaMemcpyAsync(x.p, x_init.p, xb, cudaMemcpyDeviceToDevice, stream), "restore"))) return rc;
            if ((rc = cuda(cudaMemcpyAsync(G.p, G_init.p, gb, cudaMemcpyDeviceToDevice, stream), "restore"))) return rc;
            if ((rc = cuda(cudaMemcpyAsync(carry.p, carry_init.p, cb, cudaMemcpyDeviceToDevice, stream), "restore")))
                return rc;
            if ((rc = cuda(cudaMemsetAsync(t.p, 0, tb, stream), "restore"))) return rc;
            return cuda(cudaMemcpyAsync(sv.p, sv_init.p, sb, cudaMemcpyDeviceToDevice, stream), "restore");
        }
        auto at = [](const Buf &b, size_t bytes, int64_t k) { return (char *)b.p + bytes * (size_t)k; };
        if ((rc = cuda(cudaMemcpyAsync(x.p, at(ck_x, xb, k), xb, cudaMemcpyDeviceToDevice, stream), "restore")))
            return rc;
        if ((rc = cuda(cudaMemcpyAsync(G.p, at(ck_G, gb, k), gb, cudaMemcpyDeviceToDevice, stream), "restore")))
            return rc;
        if ((rc = cuda(cudaMemcpyAsync(carry.p, at(ck_carry, cb, k), cb, cudaMemcpyDeviceToDevice, stream), "restore")))
            return rc;
        if ((rc = cuda(cudaMemcpyAsync(t.p, at(ck_t, tb, k), tb, cudaMemcpyDeviceToDevice, stream), "restore")))
            return rc;
        return cuda(cudaMemcpyAsync(sv.p, at(ck_sv, sb, k), sb, cudaMemcpyDeviceToDevice, stream), "restore");
    }
    int save(int64_t k) {
        const size_t xb = sizeof(CruD) * n_crus, gb = sizeof(double) * kNumGlobals * n_cells;
        const size_t cb = sizeof(double) * 4 * n_cells, tb = sizeof(double) * n_cells;
        const size_t sb = sizeof(double) * kSvCount * n_cells;
        auto at = [](const Buf &b, size_t bytes, int64_t k) { return (char *)b.p + bytes * (size_t)k; };
        int rc;
        if ((rc = cuda(cudaMemcpyAsync(at(ck_x, xb, k), x.p, xb, cudaMemcpyDeviceToDevice, stream), "checkpoint")))
            return rc;
        if ((rc = cuda(cudaMemcpyAsync(at(ck_G, gb, k), G.p, gb, cudaMemcpyDeviceToDevice, stream), "checkpoint")))
            return rc;
        if ((rc = cuda(cudaMemcpyAsync(at(ck_carry, cb, k), carry.p, cb, cudaMemcpyDeviceToDevice, stream),
                       "checkpoint")))
            return rc;
        if ((rc = cuda(cudaMemcpyAsync(at(ck_t, tb, k), t.p, tb, cudaMemcpyDeviceToDevice, stream), "checkpoint")))
            return rc;
        return cuda(cudaMemcpyAsync(at(ck_sv, sb, k), sv.p, sb, cudaMemcpyDeviceToDevice, stream), "checkpoint");
    }
    int check_status(const Buf &st, int n, const char *what) {
        std::vector<int> s(n);
        int rc = cuda(cudaMemcpyAsync(s.data(), st.p, sizeof(int) * n, cudaMemcpyDeviceToHost, stream), what);
        if (rc) return rc;
        if ((rc = cuda(cudaStreamSynchronize(stream), what))) return rc;
        for (int c = 0; c < n; ++c)
            if (s[c] != 0)
                return fail_to(err, s[c], "%s: cell %d stopped with status %d (%s)", what, c, s[c],
                               s[c] == GW_ERR_NERNST      ? "non-positive Nernst argument"
                               : s[c] == GW_ERR_NONFINITE ? "non-finite global state"
                                                          : "jump cap exceeded");
        return GW_OK;
    }
};

extern "C" {

int gw_grad_create(const gw_grad_desc *d, gw_grad **out) {
    g_grad_create_error.clear();
    if (!out) return fail_to(g_grad_create_error, GW_ERR_INVALID_ARGUMENT, "null output pointer");
    *out = nullptr;
    if (!d || d->n_cells < 1 || !d->ncru || !d->params || !d->stim)
        return fail_to(g_grad_create_error, GW_ERR_INVALID_ARGUMENT, "null descriptor field or n_cells < 1");
    if (!(d->dt > 0.0) || d->n_steps < 1 || d->sample_every < 1 || d->checkpoint_every < 0 || d->event_cap < 0)
        return fail_to(g_grad_create_error, GW_ERR_INVALID_ARGUMENT,
                       "need dt > 0, n_steps >= 1, sample_every >= 1, checkpoint_every >= 0, event_cap >= 0");
    if (d->cell_base < 0 || (int64_t)d->cell_base + d->n_cells > (int64_t)(1 << 28))
        return fail_to(g_grad_create_error, GW_ERR_INVALID_ARGUMENT,
                       "need 0 <= cell_base and cell_base + n_cells <= 2^28");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail_to(g_grad_create_error, GW_ERR_NO_DEVICE, "no CUDA device");
    }
    if (d->device < 0 || d->device >= ndev)
        return fail_to(g_grad_create_error, GW_ERR_INVALID_ARGUMENT, "device %d of %d", d->device, ndev);
    int major = 0, minor = 0;
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, d->device);
    cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, d->device);
    if (major != 10 || minor != 3)
        return fail_to(g_grad_create_error, GW_ERR_NO_DEVICE, "device %d is sm_%d%d; this build targets sm_103a",
                       d->device, major, minor);
    cudaSetDevice(d->device);
    gw_grad *g = new gw_grad;
    g->device = d->device;
    g->n_cells = d->n_cells;
    g->dt = d->dt;
    g->n_steps = d->n_steps;
    g->sample_every = d->sample_every;
    g->n_samples = d->n_steps / d->sample_every;
    g->ck_every = d->checkpoint_every > 0 ? d->checkpoint_every : 200;
    g->n_ck = (d->n_steps + g->ck_every - 1) / g->ck_every;
    g->event_cap = d->event_cap > 0 ? d->event_cap : 65536;
    g->seed = d->seed;
    g->cell_base = d->cell_base;
    g->stim.assign(d->stim, d->stim + 4 * (size_t)d->n_cells);
    g->have_state.assign(d->n_cells, 0);
    g->cs.resize(d->n_cells);
    g->ncru.resize(d->n_cells);
    g->cru0.resize(d->n_cells);
    for (int c = 0; c < d->n_cells; ++c) {
        const int n = d->ncru[c];
        if (n < 1) {
            delete g;
            return fail_to(g_grad_create_error, GW_ERR_INVALID_ARGUMENT, "cell %d: ncru %d < 1", c, n);
        }
        g->ncru[c] = n;
        g->cru0[c] = g->n_crus;
        g->n_crus += n;
        make_cell_static(d->params[d->params_per_cell ? c : 0], n, g->cs[c]);
        g->cru_cell.insert(g->cru_cell.end(), (size_t)n, c);
    }
    {
        int per_sm = 1;
        cudaDeviceGetAttribute(&g->sm_count, cudaDevAttrMultiProcessorCount, d->device);
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_ssa<false>, kBlk, 0) != cudaSuccess) {
            cudaGetLastError();
            per_sm = 1;
        }
        g->slots = std::max(1, g->sm_count * std::max(1, per_sm));
    }
    plan_blocks(g->ncru, g->slots, g->blk_cell, g->blk_lo, g->blk_hi, g->blk0);
    {
        // the engine's global-step program (one for all cells) and its per-cell constants
        bool pow_fast = true;
        for (int c = 0; c < d->n_cells; ++c) pow_fast = pow_fast && g->cs[c].p.Hf == 0.75 && g->cs[c].p.Hr == 0.75;
        for (int c = 0; c < d->n_cells; ++c)
            if (!ode_program_build(g->cs[c], pow_fast, c == 0 ? &g->prog : nullptr, g->cs[c].ode_consts)) {
                delete g;
                return fail_to(g_grad_create_error, GW_ERR_UNSUPPORTED, "global-step program does not fit its tables");
            }
    }
    g->n_blocks = (int)g->blk_cell.size();
    std::vector<int> rng_cell(d->n_cells);
    for (int c = 0; c < d->n_cells; ++c) rng_cell[c] = d->cell_base + c;
    const int64_t C = d->n_cells, N = g->n_crus, S = g->ck_every, K = g->n_ck;
    int rc = 0;
    auto up = [&](Buf &b, const void *src, size_t bytes) {
        if (rc) return;
        rc = g->alloc(b, bytes, "gw_grad_create");
        if (!rc && src) rc = g->cuda(cudaMemcpy(b.p, src, bytes, cudaMemcpyHostToDevice), "gw_grad_create");
    };
    up(g->d_cs, g->cs.data(), sizeof(CellStatic) * C);
    up(g->d_prog, &g->prog, sizeof(OdeProgram));
    up(g->d_blk_cell, g->blk_cell.data(), sizeof(int) * g->n_blocks);
    up(g->d_blk_lo, g->blk_lo.data(), sizeof(int) * g->n_blocks);
    up(g->d_blk_hi, g->blk_hi.data(), sizeof(int) * g->n_blocks);
    up(g->d_blk0, g->blk0.data(), sizeof(int) * (C + 1));
    up(g->part, nullptr, sizeof(double) * 4 * g->n_blocks);
    up(g->ai_part, nullptr, sizeof(double) * kAdjIn * g->n_blocks);
    up(g->d_cru_cell, g->cru_cell.data(), sizeof(int) * N);
    up(g->d_cc, nullptr, sizeof(dev::SsaConsts<double>) * C);
    up(g->d_cru0, g->cru0.data(), sizeof(int64_t) * C);
    up(g->d_ncru, g->ncru.data(), sizeof(int) * C);
    up(g->d_rng_cell, rng_cell.data(), sizeof(int) * C);
    up(g->d_stim, g->stim.data(), sizeof(double) * 4 * C);
    up(g->x_init, nullptr, sizeof(CruD) * N);
    up(g->G_init, nullptr, sizeof(double) * kNumGlobals * C);
    up(g->carry_init, nullptr, sizeof(double) * 4 * C);
    up(g->sv_init, nullptr, sizeof(double) * kSvCount * C);
    up(g->x, nullptr, sizeof(CruD) * N);
    up(g->out, nullptr, sizeof(double) * 4 * N);
    up(g->G, nullptr, sizeof(double) * kNumGlobals * C);
    up(g->carry, nullptr, sizeof(double) * 4 * C);
    up(g->t, nullptr, sizeof(double) * C);
    up(g->sv, nullptr, sizeof(double) * kSvCount * C);
    up(g->status, nullptr, sizeof(int) * C);
    up(g->events, nullptr, sizeof(unsigned long long) * C);
    up(g->V, nullptr, sizeof(double) * std::max<int64_t>(1, g->n_samples) * C);
    up(g->regime, nullptr, sizeof(unsigned long long) * C);
    up(g->ck_x, nullptr, sizeof(CruD) * N * K);
    up(g->ck_G, nullptr, sizeof(double) * kNumGlobals * C * K);
    up(g->ck_carry, nullptr, sizeof(double) * 4 * C * K);
    up(g->ck_t, nullptr, sizeof(double) * C * K);
    up(g->ck_sv, nullptr, sizeof(double) * kSvCount * C * K);
    up(g->seg_x, nullptr, sizeof(CruD) * N * S);
    up(g->seg_G, nullptr, sizeof(double) * kNumGlobals * C * S);
    up(g->seg_carry, nullptr, sizeof(double) * 4 * C * S);
    up(g->seg_sv, nullptr, sizeof(double) * kSvCount * C * S);
    up(g->quiet, nullptr, sizeof(uint8_t) * N * S);
    up(g->busy, nullptr, sizeof(int) * N * S);
    up(g->busy_n, nullptr, sizeof(int) * S);
    up(g->lam_x, nullptr, sizeof(double) * kLamX * N);
    up(g->lam_G, nullptr, sizeof(double) * kNumGlobals * C);
    up(g->lam_cy, nullptr, sizeof(double) * 3 * C);
    up(g->lam_th, nullptr, sizeof(double) * kTheta * C);
    up(g->ai_row, nullptr, sizeof(double) * kAdjIn * N);
    up(g->dLdV, nullptr, sizeof(double) * std::max<int64_t>(1, g->n_samples) * C);
    if (!rc) rc = g->cuda(cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking), "gw_grad_create");
    if (!rc) rc = g->cuda(cudaEventCreate(&g->ev0), "gw_grad_create");
    if (!rc) rc = g->cuda(cudaEventCreate(&g->ev1), "gw_grad_create");
    if (!rc) {
        k_init_consts<<<(d->n_cells + 127) / 128, 128, 0, g->stream>>>(g->d_cs.as<CellStatic>(),
                                                                      g->d_cc.as<dev::SsaConsts<double>>(), d->n_cells);
        rc = g->cuda(cudaGetLastError(), "gw_grad_create");
        if (!rc) rc = g->cuda(cudaStreamSynchronize(g->stream), "gw_grad_create");
    }
    if (rc) {
        g_grad_create_error = g->err;
        delete g;
        return rc;
    }
    g->stats.checkpoint_bytes = (int64_t)(g->ck_x.n + g->ck_G.n + g->ck_carry.n + g->ck_t.n + g->ck_sv.n);
    g->stats.segment_bytes =
        (int64_t)(g->seg_x.n + g->seg_G.n + g->seg_carry.n + g->seg_sv.n + g->quiet.n + g->busy.n + g->busy_n.n);
    *out = g;
    return GW_OK;
}

int gw_grad_destroy(gw_grad *g) {
    if (!g) return GW_OK;
    cudaSetDevice(g->device);
    delete g;
    return GW_OK;
}

int gw_grad_set_state(gw_grad *g, int cell, const gw_globals *globals, const double *CaSS, const double *CaJSR,
                      const int32_t *LCC, const int32_t *LCC_inactivation, const int32_t *RyR, const int32_t *ClCh) {
    if (!g) return GW_ERR_INVALID_ARGUMENT;
    if (cell < 0 || cell >= g->n_cells) return fail_to(g->err, GW_ERR_INVALID_ARGUMENT, "cell %d of %d", cell, g->n_cells);
    if (!globals || !CaSS || !CaJSR || !LCC || !LCC_inactivation || !RyR || !ClCh)
        return fail_to(g->err, GW_ERR_INVALID_ARGUMENT, "null state array");
    cudaSetDevice(g->device);
    const int n = g->ncru[cell];
    std::vector<CruD> xs(n);
    double clch = 0.0;
    for (int i = 0; i < n; ++i)
        if (pack_cru(CaSS, CaJSR, LCC, LCC_inactivation, RyR, ClCh, i, xs[i], clch))
            return fail_to(g->err, GW_ERR_INVALID_ARGUMENT,
                           "CRU %d: LCC not in 1..12, LCC_inactivation/ClCh not 0/1 or RyR count out of int8 range", i);
    double G0[kNumGlobals];
    std::memcpy(G0, globals, sizeof G0);
    double cy[4] = {0.0, clch, 0.0, 0.0};
    ctor_flux_carry(g->cs[cell].p, n, cy[2], cy[3]);
    double sv0[kSvCount];
    step_values(g->cs[cell], G0, sv0);
    int rc;
    if ((rc = g->cuda(cudaMemcpy(g->x_init.as<CruD>() + g->cru0[cell], xs.data(), sizeof(CruD) * n,
                                 cudaMemcpyHostToDevice), "gw_grad_set_state")))
        return rc;
    if ((rc = g->cuda(cudaMemcpy(g->G_init.as<double>() + kNumGlobals * cell, G0, sizeof G0, cudaMemcpyHostToDevice),
                      "gw_grad_set_state")))
        return rc;
    if ((rc = g->cuda(cudaMemcpy(g->carry_init.as<double>() + 4 * cell, cy, sizeof cy, cudaMemcpyHostToDevice),
                      "gw_grad_set_state")))
        return rc;
    if ((rc = g->cuda(cudaMemcpy(g->sv_init.as<double>() + kSvCount * cell, sv0, sizeof sv0, cudaMemcpyHostToDevice),
                      "gw_grad_set_state")))
        return rc;
    g->have_state[cell] = 1;
    g->forwarded = false;
    return GW_OK;
}

int gw_grad_forward(gw_grad *g, double *V_samples) {
    if (!g) return GW_ERR_INVALID_ARGUMENT;
    for (int c = 0; c < g->n_cells; ++c)
        if (!g->have_state[c]) return fail_to(g->err, GW_ERR_INVALID_ARGUMENT, "cell %d has no state", c);
    cudaSetDevice(g->device);
    int rc;
    if ((rc = g->restore(-1))) return rc;
    if ((rc = g->cuda(cudaMemsetAsync(g->status.p, 0, g->status.n, g->stream), "gw_grad_forward"))) return rc;
    if ((rc = g->cuda(cudaMemsetAsync(g->events.p, 0, g->events.n, g->stream), "gw_grad_forward"))) return rc;
    if ((rc = g->cuda(cudaMemsetAsync(g->regime.p, 0, g->regime.n, g->stream), "gw_grad_forward"))) return rc;
    if ((rc = g->cuda(cudaMemsetAsync(g->V.p, 0, g->V.n, g->stream), "gw_grad_forward"))) return rc;
    GradArgs a = g->args();
    cudaEventRecord(g->ev0, g->stream);
    for (int64_t s = 0; s < g->n_steps; ++s) {
        if (s % g->ck_every == 0 && (rc = g->save(s / g->ck_every))) return rc;
        k_ssa<false><<<g->n_blocks, kBlk, 0, g->stream>>>(a, s, 0);
        k_global<<<g->n_cells, kOdeLanes, global_layout().total, g->stream>>>(a, s, 0, 0);
    }
    cudaEventRecord(g->ev1, g->stream);
    if ((rc = g->cuda(cudaGetLastError(), "gw_grad_forward launch"))) return rc;
    if ((rc = g->check_status(g->status, g->n_cells, "gw_grad_forward"))) return rc;
    float ms = 0.f;
    if ((rc = g->cuda(cudaEventElapsedTime(&ms, g->ev0, g->ev1), "gw_grad_forward"))) return rc;
    g->stats.forward_ms = ms;
    std::vector<unsigned long long> ev(g->n_cells);
    if ((rc = g->cuda(cudaMemcpy(ev.data(), g->events.p, g->events.n, cudaMemcpyDeviceToHost), "gw_grad_forward")))
        return rc;
    g->stats.events = 0;
    for (auto e : ev) g->stats.events += (int64_t)e;
    g->G_final.resize((size_t)kNumGlobals * g->n_cells);
    if ((rc = g->cuda(cudaMemcpy(g->G_final.data(), g->G.p, g->G.n, cudaMemcpyDeviceToHost), "gw_grad_forward")))
        return rc;
    if (V_samples && g->n_samples > 0 &&
        (rc = g->cuda(cudaMemcpy(V_samples, g->V.p, sizeof(double) * g->n_samples * g->n_cells, cudaMemcpyDeviceToHost),
                      "gw_grad_forward")))
        return rc;
    g->forwarded = true;
    return GW_OK;
}

int gw_grad_backward(gw_grad *g, const double *dL_dV, double *sens) {
    if (!g) return GW_ERR_INVALID_ARGUMENT;
    if (!g->forwarded) return fail_to(g->err, GW_ERR_INVALID_ARGUMENT, "gw_grad_backward before gw_grad_forward");
    if (!dL_dV || !sens) return fail_to(g->err, GW_ERR_INVALID_ARGUMENT, "null dL_dV or sens");
    cudaSetDevice(g->device);
    int rc;
    if (g->n_samples > 0 &&
        (rc = g->cuda(cudaMemcpy(g->dLdV.p, dL_dV, sizeof(double) * g->n_samples * g->n_cells, cudaMemcpyHostToDevice),
                      "gw_grad_backward")))
        return rc;
    for (Buf *b : {&g->lam_x, &g->lam_G, &g->lam_cy, &g->lam_th})
        if ((rc = g->cuda(cudaMemsetAsync(b->p, 0, b->n, g->stream), "gw_grad_backward"))) return rc;
    GradArgs a = g->args();
    a.events = nullptr;
    a.V = nullptr;
    a.regime = nullptr;
    a.seg_x = g->seg_x.as<CruD>();
    a.seg_G = g->seg_G.as<double>();
    a.seg_carry = g->seg_carry.as<double>();
    a.seg_sv = g->seg_sv.as<double>();
    a.quiet = g->quiet.as<uint8_t>();
    a.busy = g->busy.as<int>();
    a.busy_n = g->busy_n.as<int>();
    const AdjArgs b = g->adj_args();
    const int bgrid = 2 * g->sm_count;
    cudaEventRecord(g->ev0, g->stream);
    for (int64_t k = g->n_ck - 1; k >= 0; --k) {
        const int64_t s0 = k * g->ck_every, s1 = std::min(s0 + g->ck_every, g->n_steps);
        if ((rc = g->restore(k))) return rc;
        if ((rc = g->cuda(cudaMemsetAsync(g->busy_n.p, 0, g->busy_n.n, g->stream), "gw_grad_backward"))) return rc;
        for (int64_t s = s0; s < s1; ++s) {
            k_ssa<false><<<g->n_blocks, kBlk, 0, g->stream>>>(a, s, (int)(s - s0));
            k_global<<<g->n_cells, kOdeLanes, global_layout().total, g->stream>>>(a, s, (int)(s - s0), 0);
        }
        for (int64_t s = s1 - 1; s >= s0; --s) {
            k_cru_busy<<<bgrid, kBlk, 0, g->stream>>>(a, b, s, (int)(s - s0));
            k_cru_quiet<<<g->n_blocks, kBlk, 0, g->stream>>>(a, b, (int)(s - s0));
            k_global_adj<<<g->n_cells, kBlk, 0, g->stream>>>(a, b, s, (int)(s - s0));
        }
    }
    cudaEventRecord(g->ev1, g->stream);
    if ((rc = g->cuda(cudaGetLastError(), "gw_grad_backward launch"))) return rc;
    if ((rc = g->check_status(g->status, g->n_cells, "gw_grad_backward"))) return rc;
    float ms = 0.f;
    if ((rc = g->cuda(cudaEventElapsedTime(&ms, g->ev0, g->ev1), "gw_grad_backward"))) return rc;
    g->stats.backward_ms = ms;
    return g->cuda(cudaMemcpy(sens, g->lam_th.p, sizeof(double) * kTheta * g->n_cells, cudaMemcpyDeviceToHost),
                   "gw_grad_backward");
}

int gw_grad_replay(gw_grad *g, int n_var, const int32_t *src_cell, const gw_params *params, double *V_samples,
                   int64_t *regime_steps) {
    if (!g) return GW_ERR_INVALID_ARGUMENT;
    if (n_var < 1 || !src_cell || !params || !V_samples)
        return fail_to(g->err, GW_ERR_INVALID_ARGUMENT, "need n_var >= 1 and non-null src_cell, params, V_samples");
    for (int v = 0; v < n_var; ++v) {
        if (src_cell[v] < 0 || src_cell[v] >= g->n_cells)
            return fail_to(g->err, GW_ERR_INVALID_ARGUMENT, "variant %d: source cell %d of %d", v, src_cell[v], g->n_cells);
        if (!g->have_state[src_cell[v]])
            return fail_to(g->err, GW_ERR_INVALID_ARGUMENT, "variant %d: source cell %d has no state", v, src_cell[v]);
    }
    cudaSetDevice(g->device);
    // tables of the source copies (cell v = a copy of src_cell[v]) and the variants
    std::vector<int> ncru(n_var), bc, bl, bh, b0, rngc(n_var);
    std::vector<int64_t> c0(n_var);
    std::vector<CellStatic> vcs(n_var);
    std::vector<double> stim(4 * (size_t)n_var), vsv(kSvCount * (size_t)n_var);
    int64_t N = 0;
    for (int v = 0; v < n_var; ++v) {
        const int s = src_cell[v];
        ncru[v] = g->ncru[s];
        c0[v] = N;
        N += ncru[v];
        rngc[v] = g->cell_base + s;
        for (int k = 0; k < 4; ++k) stim[4 * v + k] = g->stim[4 * s + k];
        make_cell_static(params[v], ncru[v], vcs[v]);
    }
    // the replay's global-step program: the sources' and the variants' constants under one program
    OdeProgram rprog{};
    std::vector<CellStatic> scs(n_var);
    {
        bool pow_fast = true;
        for (int v = 0; v < n_var; ++v) {
            scs[v] = g->cs[src_cell[v]];
            pow_fast = pow_fast && scs[v].p.Hf == 0.75 && scs[v].p.Hr == 0.75 && vcs[v].p.Hf == 0.75 &&
                       vcs[v].p.Hr == 0.75;
        }
        for (int v = 0; v < n_var; ++v)
            if (!ode_program_build(scs[v], pow_fast, v == 0 ? &rprog : nullptr, scs[v].ode_consts) ||
                !ode_program_build(vcs[v], pow_fast, nullptr, vcs[v].ode_consts))
                return fail_to(g->err, GW_ERR_UNSUPPORTED, "global-step program does not fit its tables");
    }
    plan_blocks(ncru, g->slots, bc, bl, bh, b0);
    const int nb = (int)bc.size();
    // initial states: the source's
    std::vector<double> G0((size_t)kNumGlobals * g->n_cells), cy0(4 * (size_t)g->n_cells),
        sv0((size_t)kSvCount * g->n_cells);
    int rc;
    if ((rc = g->cuda(cudaMemcpy(G0.data(), g->G_init.p, g->G_init.n, cudaMemcpyDeviceToHost), "gw_grad_replay")))
        return rc;
    if ((rc = g->cuda(cudaMemcpy(cy0.data(), g->carry_init.p, g->carry_init.n, cudaMemcpyDeviceToHost), "gw_grad_replay")))
        return rc;
    if ((rc = g->cuda(cudaMemcpy(sv0.data(), g->sv_init.p, g->sv_init.n, cudaMemcpyDeviceToHost), "gw_grad_replay")))
        return rc;
    std::vector<double> G(kNumGlobals * (size_t)n_var), cy(4 * (size_t)n_var), sv(kSvCount * (size_t)n_var);
    for (int v = 0; v < n_var; ++v) {
        const int s = src_cell[v];
        std::memcpy(&G[kNumGlobals * (size_t)v], &G0[kNumGlobals * (size_t)s], sizeof(double) * kNumGlobals);
        std::memcpy(&cy[4 * (size_t)v], &cy0[4 * (size_t)s], sizeof(double) * 4);
        std::memcpy(&sv[kSvCount * (size_t)v], &sv0[kSvCount * (size_t)s], sizeof(double) * kSvCount);
        step_values(vcs[v], &G0[kNumGlobals * (size_t)s], &vsv[kSvCount * (size_t)v]);
    }
    Buf d_cs, d_vcs, d_rprog, d_bc, d_bl, d_bh, d_b0, d_part, d_vpart, d_c0, d_n, d_rng, d_stim, x, out, vx, vout, dG, dvG, dcy, dvcy, dt_, dvt, dsv, dvsv,
        dst, dvst, dV, dreg;
    auto up = [&](Buf &b, const void *src, size_t bytes) {
        if (rc) return;
        rc = g->alloc(b, bytes, "gw_grad_replay");
        if (!rc && src) rc = g->cuda(cudaMemcpy(b.p, src, bytes, cudaMemcpyHostToDevice), "gw_grad_replay");
    };
    up(d_cs, scs.data(), sizeof(CellStatic) * n_var);
    up(d_vcs, vcs.data(), sizeof(CellStatic) * n_var);
    up(d_rprog, &rprog, sizeof(OdeProgram));
    up(d_bc, bc.data(), sizeof(int) * nb);
    up(d_bl, bl.data(), sizeof(int) * nb);
    up(d_bh, bh.data(), sizeof(int) * nb);
    up(d_b0, b0.data(), sizeof(int) * (n_var + 1));
    up(d_part, nullptr, sizeof(double) * 4 * nb);
    up(d_vpart, nullptr, sizeof(double) * 4 * nb);
    up(d_c0, c0.data(), sizeof(int64_t) * n_var);
    up(d_n, ncru.data(), sizeof(int) * n_var);
    up(d_rng, rngc.data(), sizeof(int) * n_var);
    up(d_stim, stim.data(), sizeof(double) * 4 * n_var);
    up(x, nullptr, sizeof(CruD) * N);
    up(out, nullptr, sizeof(double) * 4 * N);
    up(vx, nullptr, sizeof(double) * kLamX * N);
    up(vout, nullptr, sizeof(double) * 4 * N);
    up(dG, G.data(), sizeof(double) * kNumGlobals * n_var);
    up(dvG, G.data(), sizeof(double) * kNumGlobals * n_var);
    up(dcy, cy.data(), sizeof(double) * 4 * n_var);
    up(dvcy, cy.data(), sizeof(double) * 4 * n_var);
    up(dt_, nullptr, sizeof(double) * n_var);
    up(dvt, nullptr, sizeof(double) * n_var);
    up(dsv, sv.data(), sizeof(double) * kSvCount * n_var);
    up(dvsv, vsv.data(), sizeof(double) * kSvCount * n_var);
    up(dst, nullptr, sizeof(int) * n_var);
    up(dvst, nullptr, sizeof(int) * n_var);
    up(dV, nullptr, sizeof(double) * std::max<int64_t>(1, g->n_samples) * n_var);
    up(dreg, nullptr, sizeof(unsigned long long) * n_var);
    if (rc) return rc;
    // CRU states of the sources, and the variants' continuous part of them
    {
        std::vector<CruD> xs(g->n_crus), xr(N);
        if ((rc = g->cuda(cudaMemcpy(xs.data(), g->x_init.p, g->x_init.n, cudaMemcpyDeviceToHost), "gw_grad_replay")))
            return rc;
        std::vector<double> xv(kLamX * (size_t)N);
        for (int v = 0; v < n_var; ++v)
            for (int m = 0; m < ncru[v]; ++m) {
                const CruD &c = xs[g->cru0[src_cell[v]] + m];
                xr[c0[v] + m] = c;
                double *p = &xv[kLamX * (size_t)(c0[v] + m)];
                for (int j = 0; j < 4; ++j) {
                    p[j] = c.cass[j];
                    p[5 + j] = c.jlcc[j];
                }
                p[4] = c.cajsr;
            }
        if ((rc = g->cuda(cudaMemcpy(x.p, xr.data(), x.n, cudaMemcpyHostToDevice), "gw_grad_replay"))) return rc;
        if ((rc = g->cuda(cudaMemcpy(vx.p, xv.data(), vx.n, cudaMemcpyHostToDevice), "gw_grad_replay"))) return rc;
    }
    GradArgs a{};
    a.prog = d_rprog.as<OdeProgram>();
    a.cs = d_cs.as<CellStatic>();
    a.blk_cell = d_bc.as<int>();
    a.blk_lo = d_bl.as<int>();
    a.blk_hi = d_bh.as<int>();
    a.blk0 = d_b0.as<int>();
    a.part = d_part.as<double>();
    a.var_part = d_vpart.as<double>();
    a.cru0 = d_c0.as<int64_t>();
    a.ncru = d_n.as<int>();
    a.rng_cell = d_rng.as<int>();
    a.x = x.as<CruD>();
    a.out = out.as<double>();
    a.G = dG.as<double>();
    a.carry = dcy.as<double>();
    a.t = dt_.as<double>();
    a.sv = dsv.as<double>();
    a.stim = d_stim.as<double>();
    a.status = dst.as<int>();
    a.n_samples = g->n_samples;
    a.sample_every = g->sample_every;
    a.seed = g->seed;
    a.dt = g->dt;
    a.event_cap = g->event_cap;
    a.n_cells = n_var;
    a.n_crus = N;
    a.var_cs = d_vcs.as<CellStatic>();
    a.var_x = vx.as<double>();
    a.var_out = vout.as<double>();
    a.var_sv = dvsv.as<double>();
    // the variants' global step: the same kernel on the variant arrays
    GradArgs va = a;
    va.G = dvG.as<double>();
    va.carry = dvcy.as<double>();
    va.t = dvt.as<double>();
    va.status = dvst.as<int>();
    va.V = dV.as<double>();
    va.regime = dreg.as<unsigned long long>();
    cudaEventRecord(g->ev0, g->stream);
    for (int64_t s = 0; s < g->n_steps; ++s) {
        k_ssa<true><<<nb, kBlk, 0, g->stream>>>(a, s, 0);
        k_global<<<n_var, kOdeLanes, global_layout().total, g->stream>>>(a, s, 0, 0);
        k_global<<<n_var, kOdeLanes, global_layout().total, g->stream>>>(va, s, 0, 1);
    }
    cudaEventRecord(g->ev1, g->stream);
    if ((rc = g->cuda(cudaGetLastError(), "gw_grad_replay launch"))) return rc;
    if ((rc = g->check_status(dst, n_var, "gw_grad_replay (source copy)"))) return rc;
    if ((rc = g->check_status(dvst, n_var, "gw_grad_replay (variant)"))) return rc;
    float ms = 0.f;
    if ((rc = g->cuda(cudaEventElapsedTime(&ms, g->ev0, g->ev1), "gw_grad_replay"))) return rc;
    g->stats.replay_ms = ms;
    if (g->n_samples > 0 &&
        (rc = g->cuda(cudaMemcpy(V_samples, dV.p, sizeof(double) * g->n_samples * n_var, cudaMemcpyDeviceToHost),
                      "gw_grad_replay")))
        return rc;
    if (regime_steps) {
        std::vector<unsigned long long> r(n_var);
        if ((rc = g->cuda(cudaMemcpy(r.data(), dreg.p, dreg.n, cudaMemcpyDeviceToHost), "gw_grad_replay"))) return rc;
        for (int v = 0; v < n_var; ++v) regime_steps[v] = (int64_t)r[v];
    }
    return GW_OK;
}

int gw_grad_regime_steps(gw_grad *g, int64_t *regime_steps) {
    if (!g || !regime_steps) return GW_ERR_INVALID_ARGUMENT;
    if (!g->forwarded) return fail_to(g->err, GW_ERR_INVALID_ARGUMENT, "no forward pass yet");
    cudaSetDevice(g->device);
    std::vector<unsigned long long> r(g->n_cells);
    const int rc = g->cuda(cudaMemcpy(r.data(), g->regime.p, g->regime.n, cudaMemcpyDeviceToHost), "gw_grad_regime_steps");
    if (rc) return rc;
    for (int c = 0; c < g->n_cells; ++c) regime_steps[c] = (int64_t)r[c];
    return GW_OK;
}

int gw_grad_get_globals(gw_grad *g, int cell, gw_globals *out) {
    if (!g || !out) return GW_ERR_INVALID_ARGUMENT;
    if (cell < 0 || cell >= g->n_cells) return fail_to(g->err, GW_ERR_INVALID_ARGUMENT, "cell %d of %d", cell, g->n_cells);
    if (!g->forwarded) return fail_to(g->err, GW_ERR_INVALID_ARGUMENT, "no forward pass yet");
    std::memcpy(out, &g->G_final[(size_t)kNumGlobals * cell], sizeof(double) * kNumGlobals);
    return GW_OK;
}

int gw_grad_get_stats(gw_grad *g, gw_grad_stats *s) {
    if (!g || !s) return GW_ERR_INVALID_ARGUMENT;
    *s = g->stats;
    return GW_OK;
}

int gw_grad_last_error(gw_grad *g, char *msg, size_t len) {
    if (!msg || len == 0) return GW_ERR_INVALID_ARGUMENT;
    const std::string &e = g ? g->err : g_grad_create_error;
    std::snprintf(msg, len, "%s", e.c_str());
    return GW_OK;
}

int gw_grad_check_global(const gw_params *p, int nCRU, const double *G, const double *carry, double Istim, double dt,
                         const double *lam, double *d, double *lam_G, double *lam_carry, double *lam_theta) {
    if (!p || nCRU < 1 || !G || !carry || !lam || !d || !lam_G || !lam_carry || !lam_theta)
        return GW_ERR_INVALID_ARGUMENT;
    CellStatic C;
    make_cell_static(*p, nCRU, C);
    const Carry cy{carry[0], carry[1], carry[2], carry[3]};
    if (!glob_increment(C, G, cy, Istim, dt, d)) return GW_ERR_NERNST;
    for (int k = 0; k < kNumGlobals; ++k) lam_G[k] = 0.0;
    for (int k = 0; k < 3; ++k) lam_carry[k] = 0.0;
    for (int k = 0; k < kTheta; ++k) lam_theta[k] = 0.0;
    glob_increment_adj(C, G, cy, dt, lam, lam_G, lam_carry, lam_theta);
    return GW_OK;
}

int gw_grad_check_cru(const gw_params *p, int nCRU, const double *x, const int32_t *open, const double *in, int n_sub,
                      const double *h, const int32_t *ev, const int32_t *sub, const int32_t *onew, const double *lam_x,
                      const double *lam_carry, double *x_out, double *carry_out, double *lam_x0, double *lam_in,
                      double *lam_par) {
    if (!p || nCRU < 1 || !x || !open || !in || n_sub < 1 || !h || !ev || !sub || !onew || !lam_x || !lam_carry ||
        !x_out || !carry_out || !lam_x0 || !lam_in || !lam_par)
        return GW_ERR_INVALID_ARGUMENT;
    for (int k = 0; k < n_sub; ++k)
        if (ev[k] < EV_NONE || ev[k] > EV_JREL || sub[k] < 0 || sub[k] > 3) return GW_ERR_INVALID_ARGUMENT;
    CellStatic C;
    make_cell_static(*p, nCRU, C);
    const CruPar P = cru_par(C);
    const CruIn ci{in[0], in[1], in[2], in[3]};
    int o[4];
    CruCont s0;
    for (int j = 0; j < 4; ++j) {
        o[j] = open[j];
        s0.c[j] = x[j];
        s0.L[j] = x[5 + j];
    }
    s0.J = x[4];
    // forward, keeping every sub-step's start state
    std::vector<CruCont> st(n_sub);
    CruCont s = s0;
    cru_begin(s, o, P);
    double jt = 0.0, jx = 0.0;
    for (int k = 0; k < n_sub; ++k) {
        st[k] = s;
        cru_substep(s, h[k], ci, P, jt, jx);
        cru_event(s, ev[k], sub[k], onew[k], ci, P);
    }
    for (int j = 0; j < 4; ++j) {
        x_out[j] = s.c[j];
        x_out[5 + j] = s.L[j];
    }
    x_out[4] = s.J;
    carry_out[0] = jt;
    carry_out[1] = jx;
    // reverse
    CruCont la;
    for (int j = 0; j < 4; ++j) {
        la.c[j] = lam_x[j];
        la.L[j] = lam_x[5 + j];
        la.rel[j] = 0.0;
    }
    la.J = lam_x[4];
    CruAdjIn ai{0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int k = n_sub - 1; k >= 0; --k) {
        CruCont s1 = st[k];
        double a1, a2;
        cru_substep(s1, h[k], ci, P, a1, a2);
        cru_event_adj(s1, ev[k], sub[k], onew[k], ci, P, la, ai);
        const bool last = k == n_sub - 1;
        cru_substep_adj(st[k], h[k], ci, P, last ? lam_carry[0] : 0.0, last ? lam_carry[1] : 0.0, la, ai);
    }
    cru_begin_adj(s0, o, P, la, ai);
    for (int j = 0; j < 4; ++j) {
        lam_x0[j] = la.c[j];
        lam_x0[5 + j] = la.L[j];
    }
    lam_x0[4] = la.J;
    lam_in[0] = ai.Cai;
    lam_in[1] = ai.CaNSR;
    lam_in[2] = ai.JM;
    lam_in[3] = ai.JE;
    lam_par[0] = ai.rRyR_rel;
    lam_par[1] = ai.CSQN;
    return GW_OK;
}

}  // extern "C"
