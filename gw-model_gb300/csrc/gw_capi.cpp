// gw_capi.cpp -- host runtime behind the C ABI (include/gw_gb300.h).
//
// Owns device memory for an ensemble of cells, converts between the reference's array layouts
// and the engine's SoA planes, packs cells into thread-block clusters, and drives the engine
// kernel in launches of up to steps_per_launch global steps.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <memory>
#include <vector>

#include "gw_gb300.h"
#include "gw_internal.h"
#include "gw_ode_program.h"

using namespace gw;

namespace {

constexpr double kFaraday = 96.5;   // common.hpp:9
constexpr double kGasConst = 8.314; // common.hpp:10
constexpr int kMaxSsaWarps = 12;    // + kOdeWarps ODE warps = 512 threads per CTA
constexpr int kMaxSsaWarpsFp64 = 4; // FP64: + kOdeWarps = 256 threads (the FP64 engine's launch bound)

thread_local std::string g_create_error;
// cudaMalloc calls of this library in this process (gw_stats.device_allocs); every device
// allocation goes through DevBuf::alloc or dev_alloc
std::atomic<uint64_t> g_device_allocs{0};

struct DevBuf {
    void *p = nullptr;
    size_t n = 0;
    ~DevBuf() {
        if (p) cudaFree(p);
    }
    cudaError_t alloc(size_t bytes) {
        if (p) cudaFree(p);
        p = nullptr;
        n = bytes;
        if (bytes == 0) return cudaSuccess;
        g_device_allocs.fetch_add(1, std::memory_order_relaxed);
        cudaError_t e = cudaMalloc(&p, bytes);
        if (e == cudaSuccess) e = cudaMemset(p, 0, bytes);
        return e;
    }
    template <typename T>
    T *as() const {
        return reinterpret_cast<T *>(p);
    }
};

}  // namespace

struct gw_ctx {
    int device = 0;
    int test_extra_tx = 0;  // see GWGB300_TEST_SYNC_TIMEOUT in gw_create
    int precision = GW_PRECISION_FP64;
    bool ode64 = true;
    int n_cells = 0;
    uint64_t seed = 0;
    int cell_base = 0;  // global index of cell 0 (random streams)
    int event_cap = 65536;
    int steps_per_launch = 1000;
    std::vector<int32_t> ncru;
    std::vector<int64_t> slot0;
    int64_t n_slots = 0;
    std::vector<CellStatic> cs;
    std::vector<CellDyn> dyn_host;  // staging copy
    std::vector<CtaWork> work;
    LaunchShape shape{};
    int ssa_warps = 0, tile_cap = 0, max_cta_cell = 1, n_clusters = 0;
    size_t rsize = 8;  // bytes per Real
    DevBuf d_cs, d_dyn, d_slot0, d_work, d_lcc, d_flags, d_ryr, d_cass, d_jlcc, d_cajsr, d_cajsr_lo,
        d_events, d_status;
    std::vector<DevBuf *> stim_bufs;
    DevBuf d_prog;
    OdeProgram prog;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    gw_stats stats{};
    std::string err;
    ~gw_ctx() {
        for (auto *b : stim_bufs) delete b;
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace {

int fail(gw_ctx *c, int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (c)
        c->err = buf;
    else
        g_create_error = buf;
    return code;
}

#define CK(ctx, call)                                                                          \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess)                                                                 \
            return fail(ctx, e_ == cudaErrorMemoryAllocation ? GW_ERR_OUT_OF_MEMORY : GW_ERR_CUDA, \
                        "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__);  \
    } while (0)

}  // namespace

// Constants ctor (GW_utils.tpp:67-116), FP64, reference expression order.
void gw::make_cell_static(const gw_params &p, int nCRU, CellStatic &c) {
    std::memset(&c, 0, sizeof c);
    c.p = p;
    c.RT_F = kGasConst * p.T / kFaraday;
    c.F_RT = 1.0 / c.RT_F;
    c.CRU_factor = (double)p.NCaRU / (double)nCRU;
    c.CSA_FVcyto = p.CSA / (1000 * p.Vcyto * kFaraday);
    c.VSS_Vcyto = p.VSS / p.Vcyto;
    c.Vcyto_VNSR = p.Vcyto / p.VNSR;
    c.VJSR_VNSR = p.VJSR / p.VNSR;
    c.a = p.a;
    c.gamma0 = p.gamma0;
    c.gamma0a = c.gamma0 * p.a;
    c.gamma0a2 = c.gamma0a * p.a;
    c.gamma0a3 = c.gamma0a2 * p.a;
    c.gamma0a4 = c.gamma0a3 * p.a;
    c.binv = 1.0 / p.b;
    c.omega = p.omega;
    c.omega_b = c.omega * c.binv;
    c.omega_b2 = c.omega_b * c.binv;
    c.omega_b3 = c.omega_b2 * c.binv;
    c.omega_b4 = c.omega_b3 * c.binv;
    c.BSR_const = p.KBSR * p.BSRT;
    c.BSL_const = p.KBSL * p.BSLT;
    c.VSS_VJSR = p.VSS / p.VJSR;
    c.CSQN_const = p.KCSQN * p.CSQNT;
    c.JLCC_const = 2.0e6 * p.PCaL / p.VSS;
    c.Cao_scaled = 0.341 * p.Cao;
    c.Nao3 = p.Nao * p.Nao * p.Nao;
    c.INaCa_const = 5000.0 * p.kNaCa /
                    ((p.KmNa * p.KmNa * p.KmNa + p.Nao * p.Nao * p.Nao) * (p.KmCa + p.Cao));
    c.sigma = (std::exp(p.Nao / 67.3) - 1.0) / 7.0;
    c.INaK_const = p.INaKmax * p.Ko / (p.Ko + p.KmKo);
    c.sqrtKo = std::sqrt(p.Ko);
    c.PKv14_Csc = p.PKv14 / p.Csc;
    c.Ito2_const = 1.0e9 * p.Pto2 * kFaraday * c.CRU_factor / p.CSA;
    c.IK1_const = p.Ko / (p.Ko + p.KmK1);
    c.ICaL_const = -1000.0 * (2.0 * kFaraday * p.VSS) * c.CRU_factor / p.CSA;
    c.CMDN_const = p.KCMDN * p.CMDNT;
}

// Device allocation for the other translation units (gw_adjoint.cu), counted like DevBuf's.
int gw::dev_alloc(void **p, size_t bytes) {
    *p = nullptr;
    if (bytes == 0) return (int)cudaSuccess;
    g_device_allocs.fetch_add(1, std::memory_order_relaxed);
    cudaError_t e = cudaMalloc(p, bytes);
    if (e == cudaSuccess) e = cudaMemset(*p, 0, bytes);
    return (int)e;
}

// Flux carry of the reference's ctor (GW.hpp:73-74): initialise_Jxfer / initialise_Jtr from the
// default GlobalState and the ctor's CRU constants, summed over CRUs in order.
void gw::ctor_flux_carry(const gw_params &p, int n, double &sum_jtr, double &sum_jxfer) {
    gw_globals g;
    gw_globals_default(&g);
    const double jx = p.rxfer * (1.45370e-4 - g.Cai);
    const double jt = p.rtr * (g.CaNSR - 0.908408);
    sum_jtr = 0.0;
    sum_jxfer = 0.0;
    for (int i = 0; i < n; ++i) sum_jtr += jt;
    for (int i = 0; i < 4 * n; ++i) sum_jxfer += jx;
}

namespace {

int byte_of(int v) { return v & 0xFF; }

// Launch shape: cluster size C, CRU tile per CTA and SSA warps per CTA.  A cell needs
// ceil(ncru / tile) <= C CTAs.
// The size rule: cluster size C and CTA capacity (tile) for cells of at most max_n CRUs, from the
// requested values (0 = derive).  Depends on nothing else, so contexts holding shares of an
// ensemble reach the whole ensemble's shape when given its max_n.
void shape_rule(int precision, int max_n, int cluster_req, int tile_req, int &C, int &tile) {
    C = cluster_req > 0 ? cluster_req : 0;
    tile = tile_req > 0 ? tile_req : 0;
    if (C == 0 && tile == 0 && precision == GW_PRECISION_FP64) {
        // Default FP64: the SSA is bound by the FP64 pipe (one warp instruction per ~64 cycles per
        // sub-partition), so a cell is spread over up to 16 CTAs of at most 96 CRUs: three full
        // warps per CTA on three sub-partitions.
        C = std::min(kMaxClusterCtas, std::max(1, (max_n + 95) / 96));
        tile = (max_n + C - 1) / C;
    } else if (C == 0 && tile == 0) {
        // Default: one CRU per SSA thread where possible, at most 16 CTAs per cell.
        C = 1;
        while (C < kMaxClusterCtas && (max_n + C - 1) / C > 32 * kMaxSsaWarps) C *= 2;
        tile = (max_n + C - 1) / C;
    } else if (C == 0) {
        C = std::max(1, (max_n + tile - 1) / tile);
    } else if (tile == 0) {
        tile = (max_n + C - 1) / C;
    }
    tile = std::max(32, ((tile + 31) / 32) * 32);
}

int plan_shape(gw_ctx *c, int cluster_req, int tile_req) {
    const int max_n = *std::max_element(c->ncru.begin(), c->ncru.end());
    int C = 0, tile = 0;
    shape_rule(c->precision, max_n, cluster_req, tile_req, C, tile);
    if (C > kMaxClusterCtas || C < 1) return fail(c, GW_ERR_UNSUPPORTED, "cluster size %d not in [1,16]", C);
    const int need = (max_n + tile - 1) / tile;
    if (need > C)
        return fail(c, GW_ERR_UNSUPPORTED, "a cell of %d CRUs needs %d CTAs of %d CRUs but the cluster has %d",
                    max_n, need, tile, C);
    c->ssa_warps = std::min(c->precision == GW_PRECISION_FP64 ? kMaxSsaWarpsFp64 : kMaxSsaWarps, tile / 32);
    c->tile_cap = tile;
    // Pack cells (first-fit decreasing on CTA count) into clusters of C CTAs.
    std::vector<int> order(c->n_cells);
    for (int i = 0; i < c->n_cells; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return c->ncru[a] > c->ncru[b]; });
    std::vector<int> used;                   // CTAs used per cluster
    std::vector<std::vector<int>> members;   // cells per cluster
    c->max_cta_cell = 1;
    for (int cell : order) {
        const int k = std::max(1, (c->ncru[cell] + tile - 1) / tile);
        c->max_cta_cell = std::max(c->max_cta_cell, k);
        size_t q = 0;
        for (; q < used.size(); ++q)
            if (used[q] + k <= C) break;
        if (q == used.size()) {
            used.push_back(0);
            members.emplace_back();
        }
        members[q].push_back(cell);
        used[q] += k;
    }
    c->n_clusters = (int)used.size();
    c->work.assign((size_t)c->n_clusters * C, CtaWork{-1, 0, 0, 0, 0, 0, 0, 0});
    // A cell's CRUs are split in proportion to the CTAs' SSA warps that take CRUs: the others have
    // ssa_warps + kOdeWarps, the leader ssa_warps, or none when the cell is spread over several
    // CTAs of under kLeaderFreeCrus CRUs each: the global step (~12 k cycles, on the leader's SM)
    // then sets the step, and it runs ~10 % faster without SSA warps beside it (measured on one
    // 12,500-CRU cell over 16 CTAs: 6.75 -> 6.15 us per step early in the beat, 7.52 -> 7.32 at
    // 60-160 ms).  Larger CTA loads are SSA-bound and keep the leader's share.
    constexpr int64_t kLeaderFreeCrus = 1024;
    const int64_t wo = c->ssa_warps + kOdeWarps;
    int max_count = 0;
    for (int q = 0; q < c->n_clusters; ++q) {
        int rank = 0;
        for (int cell : members[q]) {
            const int64_t n = c->ncru[cell];
            const int k = std::max(1, (int)((n + tile - 1) / tile));
            const int64_t wl = (k >= 2 && n < kLeaderFreeCrus * k) ? 0 : c->ssa_warps;
            const int64_t W = wl + (k - 1) * wo;
            auto cum = [&](int r) -> int64_t { return r == 0 ? 0 : wl + (r - 1) * wo; };
            for (int r = 0; r < k; ++r) {
                CtaWork &w = c->work[(size_t)q * C + rank + r];
                w.cell = cell;
                w.cru_begin = (int)(n * cum(r) / W);
                w.cru_count = (int)(n * cum(r + 1) / W) - w.cru_begin;
                w.rank_in_cell = r;
                w.first = rank;
                w.n_cta_cell = k;
                w.lead_warps = (int)wl;
                max_count = std::max(max_count, w.cru_count);
            }
            rank += k;
        }
    }
    c->tile_cap = std::max(32, (max_count + 31) / 32 * 32);
    c->shape.cluster = C;
    c->shape.threads = (c->ssa_warps + kOdeWarps) * 32;
    c->shape.ctas = c->n_clusters * C;
    c->shape.smem = c->precision == GW_PRECISION_FP64
                        ? smem_bytes_fp64(c->tile_cap, c->max_cta_cell)
                        : smem_bytes_fp32(c->tile_cap, c->max_cta_cell);
    int dev_smem = 0;
    cudaDeviceGetAttribute(&dev_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device);
    if ((int)c->shape.smem > dev_smem)
        return fail(c, GW_ERR_UNSUPPORTED, "shared memory %zu B per CTA exceeds %d B", c->shape.smem, dev_smem);
    return GW_OK;
}

KernelArgs base_args(gw_ctx *c) {
    KernelArgs a;
    std::memset(&a, 0, sizeof a);
    a.prog = c->d_prog.as<OdeProgram>();
    a.work = c->d_work.as<CtaWork>();
    a.cs = c->d_cs.as<CellStatic>();
    a.dyn = c->d_dyn.as<CellDyn>();
    a.slot0 = c->d_slot0.as<int64_t>();
    a.n_slots = c->n_slots;
    a.lcc = c->d_lcc.as<uint32_t>();
    a.flags = c->d_flags.as<uint32_t>();
    a.ryr = c->d_ryr.as<uint32_t>();
    a.cass = c->d_cass.p;
    a.jlcc = c->d_jlcc.p;
    a.cajsr = c->d_cajsr.p;
    a.cajsr_lo = c->d_cajsr_lo.as<float>();
    a.seed = c->seed;
    a.cell_base = c->cell_base;
    a.event_cap = c->event_cap;
    a.n_cells = c->n_cells;
    a.events = c->d_events.as<unsigned long long>();
    a.status = c->d_status.as<int>();
    a.ssa_warps = c->ssa_warps;
    a.tile_cap = c->tile_cap;
    a.test_extra_tx = c->test_extra_tx;
    a.max_cta_cell = c->max_cta_cell;
    a.tr_cell = -1;
    return a;
}

int check_cell(gw_ctx *c, int cell) {
    if (!c) return GW_ERR_INVALID_ARGUMENT;
    if (cell < 0 || cell >= c->n_cells) return fail(c, GW_ERR_INVALID_ARGUMENT, "cell %d out of range", cell);
    return GW_OK;
}

int pull_dyn(gw_ctx *c) {
    CK(c, cudaMemcpy(c->dyn_host.data(), c->d_dyn.p, sizeof(CellDyn) * c->n_cells, cudaMemcpyDeviceToHost));
    return GW_OK;
}
int push_dyn(gw_ctx *c) {
    CK(c, cudaMemcpy(c->d_dyn.p, c->dyn_host.data(), sizeof(CellDyn) * c->n_cells, cudaMemcpyHostToDevice));
    return GW_OK;
}

// Copy one plane region [slot0, slot0 + n) of a device plane array (plane stride n_slots).
template <typename T>
int plane_get(gw_ctx *c, const DevBuf &b, int plane, int64_t s0, int64_t n, T *out) {
    CK(c, cudaMemcpy(out, b.as<T>() + plane * c->n_slots + s0, sizeof(T) * n, cudaMemcpyDeviceToHost));
    return GW_OK;
}
template <typename T>
int plane_put(gw_ctx *c, DevBuf &b, int plane, int64_t s0, int64_t n, const T *in) {
    CK(c, cudaMemcpy(b.as<T>() + plane * c->n_slots + s0, in, sizeof(T) * n, cudaMemcpyHostToDevice));
    return GW_OK;
}

// ---- gw_run_noalloc: record staging in a static device array ----------------------------------
// One array per device, in the module image.  Nothing in it has to start at zero: every record
// slot the trace unpack reads was written by the engine launch just before it.
constexpr size_t kNoallocScratchBytes = GW_NOALLOC_SCRATCH_BYTES;

}  // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[GW_NOALLOC_SCRATCH_BYTES];

namespace {

// Device address of the scratch in the current device's context, looked up on every call (it
// allocates nothing once the module is loaded; an address cached across calls would go stale if
// the host application reset the device and the module were loaded again).
int noalloc_scratch(gw_ctx *c, unsigned char **out) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
        return fail(c, GW_ERR_CUDA, "cudaGetSymbolAddress(no-allocation scratch): %s", cudaGetErrorString(e));
    *out = static_cast<unsigned char *>(p);
    return GW_OK;
}

// Engine record planes -> the reference's record layouts (gw_trace), one thread per (record, CRU).
__global__ void unpack_trace_kernel(int nr, int ncr, int64_t stride, bool fp64, const uint32_t *lcc,
                                    const uint32_t *flags, const uint32_t *ryr, const void *cass,
                                    const void *cajsr, int32_t *o_lcc, int32_t *o_lcci, int32_t *o_clch,
                                    int32_t *o_ryr, double *o_cass, double *o_cajsr) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)nr * ncr) return;
    const int64_t r = idx / ncr, i = idx % ncr;
    const uint32_t w = lcc[r * stride + i], f = flags[r * stride + i];
    for (int j = 0; j < 4; ++j) {
        const int64_t o = idx * 4 + j;
        if (o_lcc) o_lcc[o] = (int32_t)((w >> (8 * j)) & 0xFFu);
        if (o_lcci) o_lcci[o] = (int32_t)((f >> j) & 1u);
        if (o_clch) o_clch[o] = (int32_t)((f >> (4 + j)) & 1u);
        if (o_ryr)
            for (int k = 0; k < 6; ++k)
                o_ryr[o * 6 + k] = (int32_t)(int8_t)((ryr[(r * 6 + k) * stride + i] >> (8 * j)) & 0xFFu);
        if (o_cass) {
            const int64_t src = (r * 4 + j) * stride + i;
            o_cass[o] = fp64 ? static_cast<const double *>(cass)[src] : (double)static_cast<const float *>(cass)[src];
        }
    }
    if (o_cajsr) {
        const int64_t src = r * stride + i;
        o_cajsr[idx] = fp64 ? static_cast<const double *>(cajsr)[src] : (double)static_cast<const float *>(cajsr)[src];
    }
}

// The reference's Python currents (GWSolution, src/model.py:46-549 and :771-899) of every record of a
// launch, one thread per (cell, record), from the staged globals [cell][rec_cap][36] and CRU sums
// [cell][rec_cap][8] (int64, Ca in 2^-40 mM).  Formulas as written there (they differ from the C++
// step in places: ECa from Cai/Cao, IKv14 with Nai - Nao, ICaL with exp(2VF/RT) and the conducting
// subunits' CaSS); NCaRU / (simulated CRUs) scales the CRU-dependent currents.
__global__ void currents_kernel(const CellStatic *cs, const double *glob, const unsigned long long *sums, int rec_cap,
                                int nr, int n_cells, double *out) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)n_cells * nr) return;
    const int cell = (int)(idx / nr), r = (int)(idx % nr);
    const double *g = glob + ((int64_t)cell * rec_cap + r) * kNumGlobals;
    const unsigned long long *sm = sums + ((int64_t)cell * rec_cap + r) * kSumFields;
    const gw_params &p = cs[cell].p;
    const double F = kFaraday, F_R = kFaraday / kGasConst, F_RT = F_R / p.T;
    const double V = g[0], Nai = g[1], Ki = g[2], Cai = g[3], CaNSR = g[4];
    const double m = g[7], h = g[8], jg = g[9], xKs = g[10], XKr = g[11 + 3], XKv43 = g[16 + 4], XKv14 = g[26 + 4];
    const double Ko = p.Ko, Nao = p.Nao, Cao = p.Cao;
    const double ENa = log(Nao / Nai) / F_RT, EK = log(Ko / Ki) / F_RT;
    const double EKs = log((Ko + 0.01833 * Nao) / (Ki + 0.01833 * Nai)) / F_RT, ECa = 0.5 * log(Cao / Cai) / F_RT;
    double *o = out + ((int64_t)cell * rec_cap + r) * GW_CURRENTS;
    o[GW_CUR_INA] = p.GNa * (m * m * m) * h * jg * (V - ENa);
    o[GW_CUR_INAB] = p.GNab * (V - ENa);
    o[GW_CUR_IKR] = 0.5 * p.GKr * sqrt(Ko) * (1.0 / (1.0 + 1.4945 * exp(0.0446 * V))) * XKr * (V - EK);
    o[GW_CUR_IKS] = p.GKs * (xKs * xKs) * (V - EKs);
    o[GW_CUR_IKV43] = p.GKv43 * XKv43 * (V - EK);
    const double VF_RT = V * F_R / p.T, eVF = exp(VF_RT);
    const double mult14 = (p.PKv14 / p.Csc) * F * VF_RT * XKv14 / (1.0 - eVF);
    o[GW_CUR_IKV14] = mult14 * ((Ki - Ko * eVF) + 0.02 * (Nai - Nao)) * 1e9;
    o[GW_CUR_ITO1] = o[GW_CUR_IKV14] + o[GW_CUR_IKV43];
    const double K1inf = 1.0 / (2.0 + exp(1.5 * (V - EK) * F_R / p.T));
    o[GW_CUR_IK1] = p.GK1 * K1inf * (Ko / (Ko + p.KmK1)) * (V - EK);
    o[GW_CUR_IKP] = p.GKp * (1.0 / (1.0 + exp((7.488 - V) / 5.98))) * (V - EK);
    const double sigma = (exp(Nao / 67.3) - 1.0) / 7.0;
    const double fNaK = 1.0 / (1.0 + 0.1245 * exp(-0.1 * V * F_R / p.T) + 0.0365 * sigma * exp(-V * F_R / p.T));
    o[GW_CUR_INAK] = p.INaKmax * Ko / (Ko + p.KmKo) * fNaK / (1.0 + pow(p.KmNai / Nai, 1.5));
    const double e1 = exp(p.eta * V * F_R / p.T), e2 = exp((p.eta - 1.0) * V * F_R / p.T);
    const double multNaCa = 5000.0 * p.kNaCa / ((p.KmNa * p.KmNa * p.KmNa + Nao * Nao * Nao) * (p.KmCa + Cao));
    o[GW_CUR_INACA] = multNaCa * (e1 * (Nai * Nai * Nai) * Cao - e2 * (Nao * Nao * Nao) * Cai) / (1.0 + p.ksat * e2);
    o[GW_CUR_IPCA] = p.IpCamax * (Cai / (p.KmpCa + Cai));
    o[GW_CUR_ICAB] = p.GCab * (V - ECa);
    const double fu = pow(Cai / p.Kmf, p.Hf), ru = pow(CaNSR / p.Kmr, p.Hr);
    o[GW_CUR_JUP] = (p.Vmaxf * fu - p.Vmaxr * ru) / (1.0 + fu + ru);
    auto S = [&](int f) {
        const long long v = (long long)sm[f];
        const bool ca = f == GW_SUM_CASS_CONDUCTING || f == GW_SUM_CASS || f == GW_SUM_CAJSR;
        return ca ? ldexp((double)v, -40) : (double)v;
    };
    const double n = S(GW_SUM_CRUS), scale = (double)p.NCaRU / n;
    const double e2VF = exp(2.0 * VF_RT);
    const double multL = scale * (p.PCaL / p.CSA) * (4.0 * F * VF_RT) / (e2VF - 1.0);
    o[GW_CUR_ICAL] = multL * (e2VF * S(GW_SUM_CASS_CONDUCTING) - 0.341 * Cao * S(GW_SUM_LCC_CONDUCTING)) * 1e9;
    const double emVF = exp(-VF_RT);
    const double multT = scale * (p.Pto2 / p.CSA) * (F * VF_RT) / (emVF - 1.0);
    o[GW_CUR_ITO2] = multT * S(GW_SUM_CLCH_OPEN) * (p.Clcyto * emVF - p.Clo) * 1e9;
    o[GW_CUR_JTR] = p.rtr * (n * CaNSR - S(GW_SUM_CAJSR));
    o[GW_CUR_JXFER] = p.rxfer * (S(GW_SUM_CASS) - 4.0 * n * Cai);
    o[GW_CUR_LCC_OPEN_FRACTION] = S(GW_SUM_LCC_OPEN) / (4.0 * n);
    o[GW_CUR_RYR_OPEN_FRACTION] = S(GW_SUM_RYR_OPEN) / (20.0 * n);
}

// Bump allocator over the scratch (256-byte aligned regions).
struct ScratchCursor {
    unsigned char *base;
    size_t used;
    template <typename T>
    T *take(size_t bytes) {
        if (bytes == 0) return nullptr;
        T *p = reinterpret_cast<T *>(base + used);
        used += (bytes + 255) & ~(size_t)255;
        return p;
    }
};

}  // namespace

extern "C" {

int gw_abi_version(void) { return GW_ABI_VERSION; }

void gw_params_default(gw_params *p) {
    // GW_utils.hpp:40-156
    *p = gw_params{310.0, 153.4, 25.84, 1.113, 22.26e-6, 0.2303e-6, 12500, 4.0, 138.0, 2.0, 150.0,
                   20.0, 0.85, 2.0, 0.005, 7.0, 2.0, 1.9356, 0.44, 0.02158, 9.13e-13, 13.3156, 2.0,
                   2.65e-15, 877.5, 250.0, 2.358e8, 9.6, 1.415e6, 13.65, 0.07, 93.385, 1.887e7,
                   30.0, 2.358e6, 0.001235, 3.92, 200.0, 0.333, 20.0, 0.047, 0.00087, 1.124,
                   0.0087, 13.5, 0.63, 0.05, 0.00238, 12.8, 0.024, 0.0266, 0.1348, 0.00271, 0.1389,
                   0.5437, 0.02898, 0.08019, 0.04684, 0.04984, 3.37302e-4, 8.1948e-4, 5.374e-8,
                   1.8936, 14.225, 158.574, 142.937, 6.7735, 15.621, 28.753, 524.576, 1.989e-7,
                   1.8931, 0.006950, 0.01179, 0.08527, 0.002963, 0.0, 1.0571e-4, 0.0, 0.2001,
                   0.3203, 13.509, 1151.765, 2.230, 12.0, 5.370, 5.240, 1.0e6, 3.0, 13.0, 0.002659,
                   0.27, 87.5, 1.38, 0.2, 0.35, 0.901, 10.0, 1.5, 0.03, 0.0005, 0.0002536, 0.00264,
                   20.0, 6.60e-5, 40.0, 0.04, 0.140, 0.070, 0.0002096, 0.0002096, 0.000260, 1.8,
                   0.75, 0.75};
}

void gw_globals_default(gw_globals *g) {
    // GW_utils.hpp:231-247
    *g = gw_globals{-91.382, 10.0, 131.84, 1.45273e-4, 0.908882, 8.98282e-3, 0.137617, 5.33837e-4,
                    0.996345, 0.997315, 2.04171e-4,
                    {0.999503, 4.13720e-4, 7.27568e-5, 8.73984e-6, 1.36159e-6},
                    {0.953060, 0.0253906, 2.53848e-4, 1.12796e-6, 1.87950e-9, 0.0151370,
                     0.00517622, 8.96600e-4, 8.17569e-5, 2.24032e-6},
                    {0.722328, 0.101971, 0.00539932, 1.27081e-4, 1.82742e-6, 0.152769, 0.00962328,
                     0.00439043, 0.00195348, 0.00143629}};
}

void gw_globals_py_default(gw_globals *g) {
    gw_globals_default(g);
    g->CaLTRPN = 8.9282e-3;  // pyGW.cpp:37
}

int gw_create(const gw_ensemble_desc *d, gw_ctx **out) {
    if (!d || !out) return fail(nullptr, GW_ERR_INVALID_ARGUMENT, "null descriptor or output");
    *out = nullptr;
    if (d->n_cells <= 0 || !d->ncru || !d->params)
        return fail(nullptr, GW_ERR_INVALID_ARGUMENT, "n_cells must be > 0 with ncru and params");
    if (d->precision != GW_PRECISION_FP64 && d->precision != GW_PRECISION_FP32)
        return fail(nullptr, GW_ERR_INVALID_ARGUMENT, "unknown precision %d", d->precision);
    for (int i = 0; i < d->n_cells; ++i)
        if (d->ncru[i] <= 0) return fail(nullptr, GW_ERR_INVALID_ARGUMENT, "cell %d: nCRU must be > 0", i);
    if (d->cell_base < 0 || (int64_t)d->cell_base + d->n_cells > (int64_t)(1 << 28))
        return fail(nullptr, GW_ERR_INVALID_ARGUMENT, "need 0 <= cell_base and cell_base + n_cells <= 2^28");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return fail(nullptr, GW_ERR_NO_DEVICE, "no CUDA device");
    if (d->device < 0 || d->device >= ndev) return fail(nullptr, GW_ERR_INVALID_ARGUMENT, "bad device %d", d->device);
    int major = 0, minor = 0;
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, d->device);
    cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, d->device);
    if (major != 10 || minor != 3)
        return fail(nullptr, GW_ERR_NO_DEVICE, "device %d is sm_%d%d; this build targets sm_103a", d->device, major, minor);
    gw_ctx *c = new gw_ctx;
    c->device = d->device;
    c->precision = d->precision;
    c->ode64 = d->precision == GW_PRECISION_FP64 || d->ode_fp32_rhs == 0;
    c->n_cells = d->n_cells;
    c->seed = d->seed;
    c->cell_base = d->cell_base;
    c->event_cap = d->event_cap > 0 ? d->event_cap : 65536;
    // Test hook for the bounded waits of the engine kernel: GWGB300_TEST_SYNC_TIMEOUT=1 at context
    // creation makes every launch's last wait for the warp partials expect 16 bytes that are never
    // sent, so that it runs out (about a second) and the launch reports GW_ERR_SYNC_TIMEOUT.
    {
        const char *t = getenv("GWGB300_TEST_SYNC_TIMEOUT");
        c->test_extra_tx = (t && t[0] == '1') ? 16 : 0;
    }
    c->steps_per_launch = d->steps_per_launch > 0 ? d->steps_per_launch : 1000;
    c->rsize = c->precision == GW_PRECISION_FP64 ? 8 : 4;
    c->ncru.assign(d->ncru, d->ncru + d->n_cells);
    if (cudaSetDevice(c->device) != cudaSuccess) {
        delete c;
        return fail(nullptr, GW_ERR_CUDA, "cudaSetDevice failed");
    }
    int rc = plan_shape(c, d->cluster_ctas, d->cta_crus);
    if (rc != GW_OK) {
        g_create_error = c->err;
        delete c;
        return rc;
    }
    c->slot0.resize(c->n_cells);
    int64_t s = 0;
    for (int i = 0; i < c->n_cells; ++i) {
        c->slot0[i] = s;
        s += ((int64_t)c->ncru[i] + 31) / 32 * 32;
    }
    c->n_slots = s;
    c->cs.resize(c->n_cells);
    c->dyn_host.assign(c->n_cells, CellDyn{});
    bool pow_fast = true;
    for (int i = 0; i < c->n_cells; ++i) {
        const gw_params &p = d->params[d->params_per_cell ? i : 0];
        pow_fast = pow_fast && p.Hf == 0.75 && p.Hr == 0.75;
    }
    for (int i = 0; i < c->n_cells; ++i) {
        const gw_params &p = d->params[d->params_per_cell ? i : 0];
        make_cell_static(p, c->ncru[i], c->cs[i]);
        if (!ode_program_build(c->cs[i], pow_fast, i == 0 ? &c->prog : nullptr, c->cs[i].ode_consts)) {
            g_create_error = "global-step program does not fit its tables";
            delete c;
            return GW_ERR_UNSUPPORTED;
        }
        CellDyn &y = c->dyn_host[i];
        std::memset(&y, 0, sizeof y);
        gw_globals g;
        gw_globals_default(&g);
        std::memcpy(y.g, &g, sizeof g);
        ctor_flux_carry(p, c->ncru[i], y.sum_jtr, y.sum_jxfer);
    }
    auto alloc_all = [&]() -> int {
        CK(c, cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
        CK(c, cudaEventCreate(&c->ev0));
        CK(c, cudaEventCreate(&c->ev1));
        CK(c, c->d_cs.alloc(sizeof(CellStatic) * c->n_cells));
        CK(c, c->d_prog.alloc(sizeof(OdeProgram)));
        CK(c, cudaMemcpy(c->d_prog.p, &c->prog, sizeof(OdeProgram), cudaMemcpyHostToDevice));
        CK(c, c->d_dyn.alloc(sizeof(CellDyn) * c->n_cells));
        CK(c, c->d_slot0.alloc(sizeof(int64_t) * c->n_cells));
        CK(c, c->d_work.alloc(sizeof(CtaWork) * c->work.size()));
        CK(c, c->d_lcc.alloc(4 * c->n_slots));
        CK(c, c->d_flags.alloc(4 * c->n_slots));
        CK(c, c->d_ryr.alloc(4 * 6 * c->n_slots));
        CK(c, c->d_cass.alloc(c->rsize * 4 * c->n_slots));
        CK(c, c->d_jlcc.alloc(c->rsize * 4 * c->n_slots));
        CK(c, c->d_cajsr.alloc(c->rsize * c->n_slots));
        CK(c, c->d_cajsr_lo.alloc(4 * c->n_slots));
        CK(c, c->d_events.alloc(sizeof(unsigned long long)));
        CK(c, c->d_status.alloc(sizeof(int) * c->n_cells));
        CK(c, cudaMemcpy(c->d_cs.p, c->cs.data(), sizeof(CellStatic) * c->n_cells, cudaMemcpyHostToDevice));
        CK(c, cudaMemcpy(c->d_slot0.p, c->slot0.data(), sizeof(int64_t) * c->n_cells, cudaMemcpyHostToDevice));
        CK(c, cudaMemcpy(c->d_work.p, c->work.data(), sizeof(CtaWork) * c->work.size(), cudaMemcpyHostToDevice));
        return GW_OK;
    };
    rc = alloc_all();
    if (rc == GW_OK) rc = push_dyn(c);
    // The reference's ctor draws a random CRU state (GW_utils.tpp:210-218); draw it here too.
    for (int i = 0; rc == GW_OK && i < c->n_cells; ++i) rc = gw_sample_initial_crus(c, i);
    if (rc == GW_OK) {
        int nclus = 0;
        const int e = c->precision == GW_PRECISION_FP64 ? max_active_clusters_fp64(c->shape, c->ode64, &nclus)
                                                        : max_active_clusters_fp32(c->shape, c->ode64, &nclus);
        if (e != 0 || nclus < 1)
            rc = fail(c, GW_ERR_UNSUPPORTED,
                      "launch shape (cluster %d x %d threads, %zu B smem) cannot be resident (err %d, %d clusters)",
                      c->shape.cluster, c->shape.threads, c->shape.smem, e, nclus);
    }
    if (rc != GW_OK) {
        g_create_error = c->err;
        delete c;
        return rc;
    }
    c->stats.cluster_ctas = c->shape.cluster;
    c->stats.cta_crus = c->tile_cap;
    c->stats.threads_per_cta = c->shape.threads;
    c->stats.n_clusters = c->n_clusters;
    c->stats.ctas = c->shape.ctas;
    *out = c;
    return GW_OK;
}

int gw_destroy(gw_ctx *c) {
    if (!c) return GW_ERR_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    delete c;
    return GW_OK;
}

int gw_default_shape(const gw_ensemble_desc *d, int *cluster_ctas, int *cta_crus) {
    if (!d || !cluster_ctas || !cta_crus || d->n_cells <= 0 || !d->ncru)
        return fail(nullptr, GW_ERR_INVALID_ARGUMENT, "gw_default_shape: null descriptor/output or n_cells <= 0");
    int max_n = 0;
    for (int i = 0; i < d->n_cells; ++i) {
        if (d->ncru[i] <= 0) return fail(nullptr, GW_ERR_INVALID_ARGUMENT, "cell %d: nCRU must be > 0", i);
        max_n = std::max(max_n, (int)d->ncru[i]);
    }
    shape_rule(d->precision, max_n, d->cluster_ctas, d->cta_crus, *cluster_ctas, *cta_crus);
    return GW_OK;
}

int gw_autotune(const gw_ensemble_desc *d, int trial_steps, int *best_cluster_ctas, int *best_cta_crus,
                double *best_us_per_step) {
    if (!d || !best_cluster_ctas || trial_steps <= 0 || d->n_cells <= 0 || !d->ncru)
        return fail(nullptr, GW_ERR_INVALID_ARGUMENT, "gw_autotune: null descriptor/output or trial_steps <= 0");
    // Cluster sizes: powers of two, and 9, 6, 3, which pack two, three and six clusters into a
    // GPC of 18-19 SMs (GB300: 152 SMs) where 8 and 4 leave SMs idle.
    static const int kCandidates[] = {16, 9, 8, 6, 4, 3, 2, 1};
    const int warm = std::max(20, trial_steps / 4);
    // The planner alone (no allocation): whether a cluster size and CTA capacity fit these cells.
    std::unique_ptr<gw_ctx> probe(new gw_ctx);
    probe->device = d->device;
    probe->precision = d->precision;
    probe->n_cells = d->n_cells;
    probe->ncru.assign(d->ncru, d->ncru + d->n_cells);
    auto fits = [&](int C, int tile) { return plan_shape(probe.get(), C, tile) == GW_OK; };
    int best = 0, best_tile = 0;
    double best_us = 0.0;
    for (int C : kCandidates) {
        if (!fits(C, 0)) continue;  // this cluster size does not fit the cells
        // Two capacities per cluster size: the size rule's, and the largest that fits shared
        // memory (fewer, fuller CTAs amortise the per-step barrier and global step over more CRUs,
        // which pays off for cells of uneven size).
        int big = 0;
        for (int t = 4096; t > 0; t -= 64)
            if (fits(C, t)) {
                big = t;
                break;
            }
        const int rule_tile = fits(C, 0) ? probe->tile_cap : 0;
        const int tiles[2] = {0, big > rule_tile + 64 ? big : -1};
        for (int tile : tiles) {
            if (tile < 0) continue;
            gw_ensemble_desc t = *d;
            t.cluster_ctas = C;
            t.cta_crus = tile;
            gw_ctx *c = nullptr;
            int rc = gw_create(&t, &c);
            if (rc == GW_ERR_UNSUPPORTED) continue;
            if (rc) return rc;
            rc = gw_set_stimulus_pulse(c, -1, 0.0, 1000.0, 0.5, 100.0);
            if (!rc) rc = gw_run(c, 1e-3, warm, 0, nullptr);
            const double ms0 = c->stats.kernel_ms;
            if (!rc) rc = gw_run(c, 1e-3, trial_steps, 0, nullptr);
            const double us = (c->stats.kernel_ms - ms0) * 1e3 / trial_steps;
            if (rc) g_create_error = c->err;
            gw_destroy(c);
            if (rc) return rc;
            if (best == 0 || us < best_us) {
                best = C;
                best_tile = tile;
                best_us = us;
            }
        }
    }
    if (best == 0) return fail(nullptr, GW_ERR_UNSUPPORTED, "gw_autotune: no cluster size fits these cells");
    *best_cluster_ctas = best;
    if (best_cta_crus) *best_cta_crus = best_tile;
    if (best_us_per_step) *best_us_per_step = best_us;
    return GW_OK;
}

int gw_sample_initial_crus(gw_ctx *c, int cell) {
    int rc = check_cell(c, cell);
    if (rc) return rc;
    cudaSetDevice(c->device);
    KernelArgs a = base_args(c);
    const int e = sample_initial_crus_dev(a, cell, c->ncru[cell], c->precision == GW_PRECISION_FP64, c->stream);
    if (e != 0) return fail(c, GW_ERR_CUDA, "initial-state kernel: %s", cudaGetErrorString((cudaError_t)e));
    CK(c, cudaStreamSynchronize(c->stream));
    // JLCC = 0 and ClCh changed: refresh the JLCC / ClCh sums of the carry.
    rc = pull_dyn(c);
    if (rc) return rc;
    std::vector<uint32_t> flags(c->ncru[cell]);
    rc = plane_get(c, c->d_flags, 0, c->slot0[cell], c->ncru[cell], flags.data());
    if (rc) return rc;
    double cl = 0;
    for (uint32_t f : flags) cl += __builtin_popcount((f >> 4) & 0xFu);
    c->dyn_host[cell].sum_clch = cl;
    c->dyn_host[cell].sum_jlcc = 0.0;
    return push_dyn(c);
}

int gw_set_globals(gw_ctx *c, int cell, const gw_globals *g) {
    int rc = check_cell(c, cell);
    if (rc) return rc;
    if (!g) return fail(c, GW_ERR_INVALID_ARGUMENT, "null globals");
    cudaSetDevice(c->device);
    if ((rc = pull_dyn(c))) return rc;
    std::memcpy(c->dyn_host[cell].g, g, sizeof *g);
    return push_dyn(c);
}

int gw_get_globals(gw_ctx *c, int cell, gw_globals *g) {
    int rc = check_cell(c, cell);
    if (rc) return rc;
    if (!g) return fail(c, GW_ERR_INVALID_ARGUMENT, "null globals");
    cudaSetDevice(c->device);
    if ((rc = pull_dyn(c))) return rc;
    std::memcpy(g, c->dyn_host[cell].g, sizeof *g);
    return GW_OK;
}

int gw_set_crus(gw_ctx *c, int cell, const double *CaSS, const double *CaJSR, const int32_t *LCC,
                const int32_t *LCCi, const int32_t *RyR, const int32_t *ClCh, const double *JLCC) {
    int rc = check_cell(c, cell);
    if (rc) return rc;
    if (!CaSS || !CaJSR || !LCC || !LCCi || !RyR || !ClCh)
        return fail(c, GW_ERR_INVALID_ARGUMENT, "null CRU array");
    cudaSetDevice(c->device);
    const int n = c->ncru[cell];
    std::vector<uint32_t> lcc(n), flags(n), ryr(6 * (size_t)n);
    double cl = 0, jl = 0;
    for (int i = 0; i < n; ++i) {
        uint32_t w = 0, f = 0;
        for (int j = 0; j < 4; ++j) {
            const int s = LCC[4 * i + j];
            if (s < 1 || s > 12) return fail(c, GW_ERR_INVALID_ARGUMENT, "CRU %d subunit %d: LCC state %d not in 1..12", i, j, s);
            const int li = LCCi[4 * i + j], ch = ClCh[4 * i + j];
            if ((li != 0 && li != 1) || (ch != 0 && ch != 1))
                return fail(c, GW_ERR_INVALID_ARGUMENT, "CRU %d subunit %d: LCC_inactivation/ClCh must be 0 or 1", i, j);
            w |= (uint32_t)byte_of(s) << (8 * j);
            f |= (uint32_t)li << j;
            f |= (uint32_t)ch << (4 + j);
            cl += ch;
            for (int k = 0; k < 6; ++k) {
                const int v = RyR[24 * i + 6 * j + k];
                if (v < -128 || v > 127) return fail(c, GW_ERR_INVALID_ARGUMENT, "RyR count %d out of int8 range", v);
                ryr[(size_t)k * n + i] |= (uint32_t)byte_of(v) << (8 * j);
            }
        }
        lcc[i] = w;
        flags[i] = f;
    }
    const int64_t s0 = c->slot0[cell];
    if ((rc = plane_put(c, c->d_lcc, 0, s0, n, lcc.data()))) return rc;
    if ((rc = plane_put(c, c->d_flags, 0, s0, n, flags.data()))) return rc;
    for (int k = 0; k < 6; ++k)
        if ((rc = plane_put(c, c->d_ryr, k, s0, n, ryr.data() + (size_t)k * n))) return rc;
    std::vector<double> jv(4 * (size_t)n, 0.0);
    if (JLCC) std::memcpy(jv.data(), JLCC, sizeof(double) * 4 * n);
    for (double v : jv) jl += v;
    if (c->precision == GW_PRECISION_FP64) {
        std::vector<double> pl(n);
        for (int j = 0; j < 4; ++j) {
            for (int i = 0; i < n; ++i) pl[i] = CaSS[4 * i + j];
            if ((rc = plane_put(c, c->d_cass, j, s0, n, pl.data()))) return rc;
            for (int i = 0; i < n; ++i) pl[i] = jv[4 * i + j];
            if ((rc = plane_put(c, c->d_jlcc, j, s0, n, pl.data()))) return rc;
        }
        if ((rc = plane_put(c, c->d_cajsr, 0, s0, n, CaJSR))) return rc;
    } else {
        std::vector<float> pl(n), lo(n);
        for (int j = 0; j < 4; ++j) {
            for (int i = 0; i < n; ++i) pl[i] = (float)CaSS[4 * i + j];
            if ((rc = plane_put(c, c->d_cass, j, s0, n, pl.data()))) return rc;
            for (int i = 0; i < n; ++i) pl[i] = (float)jv[4 * i + j];
            if ((rc = plane_put(c, c->d_jlcc, j, s0, n, pl.data()))) return rc;
        }
        for (int i = 0; i < n; ++i) {
            pl[i] = (float)CaJSR[i];
            lo[i] = (float)(CaJSR[i] - (double)pl[i]);
        }
        if ((rc = plane_put(c, c->d_cajsr, 0, s0, n, pl.data()))) return rc;
        if ((rc = plane_put(c, c->d_cajsr_lo, 0, s0, n, lo.data()))) return rc;
    }
    if ((rc = pull_dyn(c))) return rc;
    c->dyn_host[cell].sum_clch = cl;
    c->dyn_host[cell].sum_jlcc = jl;
    return push_dyn(c);
}

int gw_get_crus(gw_ctx *c, int cell, double *CaSS, double *CaJSR, int32_t *LCC, int32_t *LCCi,
                int32_t *RyR, int32_t *ClCh, double *JLCC) {
    int rc = check_cell(c, cell);
    if (rc) return rc;
    cudaSetDevice(c->device);
    CK(c, cudaStreamSynchronize(c->stream));
    const int n = c->ncru[cell];
    const int64_t s0 = c->slot0[cell];
    std::vector<uint32_t> lcc(n), flags(n), ryr(6 * (size_t)n);
    if ((rc = plane_get(c, c->d_lcc, 0, s0, n, lcc.data()))) return rc;
    if ((rc = plane_get(c, c->d_flags, 0, s0, n, flags.data()))) return rc;
    for (int k = 0; k < 6; ++k)
        if ((rc = plane_get(c, c->d_ryr, k, s0, n, ryr.data() + (size_t)k * n))) return rc;
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < 4; ++j) {
            if (LCC) LCC[4 * i + j] = (int)((lcc[i] >> (8 * j)) & 0xFF);
            if (LCCi) LCCi[4 * i + j] = (int)((flags[i] >> j) & 1);
            if (ClCh) ClCh[4 * i + j] = (int)((flags[i] >> (4 + j)) & 1);
            if (RyR)
                for (int k = 0; k < 6; ++k) RyR[24 * i + 6 * j + k] = (int)(int8_t)((ryr[(size_t)k * n + i] >> (8 * j)) & 0xFF);
        }
    if (c->precision == GW_PRECISION_FP64) {
        std::vector<double> pl(n);
        for (int j = 0; j < 4; ++j) {
            if (CaSS) {
                if ((rc = plane_get(c, c->d_cass, j, s0, n, pl.data()))) return rc;
                for (int i = 0; i < n; ++i) CaSS[4 * i + j] = pl[i];
            }
            if (JLCC) {
                if ((rc = plane_get(c, c->d_jlcc, j, s0, n, pl.data()))) return rc;
                for (int i = 0; i < n; ++i) JLCC[4 * i + j] = pl[i];
            }
        }
        if (CaJSR && (rc = plane_get(c, c->d_cajsr, 0, s0, n, CaJSR))) return rc;
    } else {
        std::vector<float> pl(n), lo(n);
        for (int j = 0; j < 4; ++j) {
            if (CaSS) {
                if ((rc = plane_get(c, c->d_cass, j, s0, n, pl.data()))) return rc;
                for (int i = 0; i < n; ++i) CaSS[4 * i + j] = pl[i];
            }
            if (JLCC) {
                if ((rc = plane_get(c, c->d_jlcc, j, s0, n, pl.data()))) return rc;
                for (int i = 0; i < n; ++i) JLCC[4 * i + j] = pl[i];
            }
        }
        if (CaJSR) {
            if ((rc = plane_get(c, c->d_cajsr, 0, s0, n, pl.data()))) return rc;
            if ((rc = plane_get(c, c->d_cajsr_lo, 0, s0, n, lo.data()))) return rc;
            for (int i = 0; i < n; ++i) CaJSR[i] = (double)pl[i] + (double)lo[i];
        }
    }
    return GW_OK;
}

int gw_set_flux_carry(gw_ctx *c, int cell, double sum_JLCC, double sum_ClCh, double sum_Jtr,
                      double sum_Jxfer) {
    int rc = check_cell(c, cell);
    if (rc) return rc;
    cudaSetDevice(c->device);
    if ((rc = pull_dyn(c))) return rc;
    c->dyn_host[cell].sum_jlcc = sum_JLCC;
    c->dyn_host[cell].sum_clch = sum_ClCh;
    c->dyn_host[cell].sum_jtr = sum_Jtr;
    c->dyn_host[cell].sum_jxfer = sum_Jxfer;
    return push_dyn(c);
}

int gw_get_flux_carry(gw_ctx *c, int cell, double *sum_JLCC, double *sum_ClCh, double *sum_Jtr,
                      double *sum_Jxfer) {
    int rc = check_cell(c, cell);
    if (rc) return rc;
    cudaSetDevice(c->device);
    if ((rc = pull_dyn(c))) return rc;
    if (sum_JLCC) *sum_JLCC = c->dyn_host[cell].sum_jlcc;
    if (sum_ClCh) *sum_ClCh = c->dyn_host[cell].sum_clch;
    if (sum_Jtr) *sum_Jtr = c->dyn_host[cell].sum_jtr;
    if (sum_Jxfer) *sum_Jxfer = c->dyn_host[cell].sum_jxfer;
    return GW_OK;
}

int gw_set_stimulus_pulse(gw_ctx *c, int cell, double start, double period, double duration,
                          double amplitude) {
    if (!c) return GW_ERR_INVALID_ARGUMENT;
    if (cell >= c->n_cells) return fail(c, GW_ERR_INVALID_ARGUMENT, "cell %d out of range", cell);
    if (!(duration >= 0.0) || !std::isfinite(start) || !std::isfinite(period) || !std::isfinite(amplitude))
        return fail(c, GW_ERR_INVALID_ARGUMENT, "bad pulse train");
    cudaSetDevice(c->device);
    int rc = pull_dyn(c);
    if (rc) return rc;
    for (int i = 0; i < c->n_cells; ++i) {
        if (cell >= 0 && i != cell) continue;
        CellDyn &y = c->dyn_host[i];
        y.stim_mode = STIM_PULSE;
        y.stim_start = start;
        y.stim_period = period;
        y.stim_dur = duration;
        y.stim_amp = amplitude;
        y.stim_samples = nullptr;
        y.stim_n = 0;
    }
    return push_dyn(c);
}

int gw_set_stimulus_samples(gw_ctx *c, int cell, const double *Istim, int64_t n) {
    if (!c) return GW_ERR_INVALID_ARGUMENT;
    if (cell >= c->n_cells) return fail(c, GW_ERR_INVALID_ARGUMENT, "cell %d out of range", cell);
    if (n < 0 || (n > 0 && !Istim)) return fail(c, GW_ERR_INVALID_ARGUMENT, "bad stimulus samples");
    cudaSetDevice(c->device);
    DevBuf *b = new DevBuf;
    c->stim_bufs.push_back(b);
    CK(c, b->alloc(sizeof(double) * (size_t)std::max<int64_t>(n, 1)));
    if (n > 0) CK(c, cudaMemcpy(b->p, Istim, sizeof(double) * n, cudaMemcpyHostToDevice));
    int rc = pull_dyn(c);
    if (rc) return rc;
    for (int i = 0; i < c->n_cells; ++i) {
        if (cell >= 0 && i != cell) continue;
        CellDyn &y = c->dyn_host[i];
        y.stim_mode = STIM_SAMPLES;
        y.stim_samples = b->as<double>();
        y.stim_n = n;
    }
    return push_dyn(c);
}

int gw_run(gw_ctx *c, double dt, int64_t n_steps, int record_every, gw_trace *tr) {
    if (!c) return GW_ERR_INVALID_ARGUMENT;
    if (!(dt > 0.0) || !std::isfinite(dt)) return fail(c, GW_ERR_INVALID_ARGUMENT, "dt must be > 0");
    if (n_steps < 0) return fail(c, GW_ERR_INVALID_ARGUMENT, "n_steps must be >= 0");
    if (record_every < 0) return fail(c, GW_ERR_INVALID_ARGUMENT, "record_every must be >= 0");
    cudaSetDevice(c->device);
    if (tr) tr->n_written = 0;
    const bool recording = tr && record_every > 0 && tr->max_records > 0;
    const bool planes = recording && (tr->CaSS || tr->CaJSR || tr->LCC || tr->LCC_inactivation || tr->RyR || tr->ClCh);
    const bool codec = recording && (tr->LCC_i8 || tr->LCC_inactivation_u8 || tr->ClCh_u8 || tr->RyR_i16 ||
                                     tr->CaSS_f32 || tr->CaJSR_f32);
    const bool currents = recording && tr->currents;
    const bool sums = recording && (tr->cru_sums || currents);
    if (planes && codec)
        return fail(c, GW_ERR_INVALID_ARGUMENT,
                    "trace: request either the int32/double CRU arrays or the reduced-memory ones, not both");
    const int tr_cell = (planes || codec) ? tr->cru_cell : -1;
    if (tr_cell >= c->n_cells) return fail(c, GW_ERR_INVALID_ARGUMENT, "trace cell out of range");
    {
        // the RNG counter holds 32 bits of the step index
        int rc = pull_dyn(c);
        if (rc) return rc;
        for (int i = 0; i < c->n_cells; ++i)
            if (c->dyn_host[i].step + (uint64_t)n_steps > 0xFFFFFFFFull)
                return fail(c, GW_ERR_INVALID_ARGUMENT, "more than 2^32 steps in one context");
    }
    const int chunk = c->steps_per_launch;
    // Device trace buffers for the records of one launch.
    const int rec_cap = recording ? (int)std::min<int64_t>(tr->max_records, chunk / record_every + 2) : 0;
    DevBuf d_t, d_glob, d_tlcc, d_tflags, d_tryr, d_tcass, d_tcajsr, d_gate, d_clch, d_ryrc, d_cassf, d_cajsrf, d_sums,
        d_cur;
    int64_t stride = 0;
    const int64_t ncr = tr_cell >= 0 ? c->ncru[tr_cell] : 0;
    if (recording) {
        CK(c, d_t.alloc(sizeof(double) * rec_cap));
        CK(c, d_glob.alloc(sizeof(double) * kNumGlobals * (size_t)rec_cap * c->n_cells));
        if (planes && tr_cell >= 0) {
            stride = (ncr + 31) / 32 * 32;
            CK(c, d_tlcc.alloc(4 * stride * rec_cap));
            CK(c, d_tflags.alloc(4 * stride * rec_cap));
            CK(c, d_tryr.alloc(4 * 6 * stride * rec_cap));
            CK(c, d_tcass.alloc(c->rsize * 4 * stride * rec_cap));
            CK(c, d_tcajsr.alloc(c->rsize * stride * rec_cap));
        }
        if (codec && tr_cell >= 0) {
            CK(c, d_tlcc.alloc(4 * ncr * rec_cap));
            CK(c, d_gate.alloc(4 * ncr * rec_cap));
            CK(c, d_clch.alloc(4 * ncr * rec_cap));
            CK(c, d_ryrc.alloc(8 * ncr * rec_cap));
            CK(c, d_cassf.alloc(16 * ncr * rec_cap));
            CK(c, d_cajsrf.alloc(4 * ncr * rec_cap));
        }
        if (sums) CK(c, d_sums.alloc(sizeof(unsigned long long) * kSumFields * (size_t)rec_cap * c->n_cells));
        if (currents) CK(c, d_cur.alloc(sizeof(double) * GW_CURRENTS * (size_t)rec_cap * c->n_cells));
    }
    KernelArgs a = base_args(c);
    a.dt = dt;
    a.record_every = recording ? record_every : 0;
    a.rec_cap = rec_cap;
    a.tr_t = d_t.as<double>();
    a.tr_glob = d_glob.as<double>();
    a.tr_cell = tr_cell;
    a.tr_cru_stride = stride;
    a.tr_lcc = d_tlcc.as<uint32_t>();
    a.tr_flags = d_tflags.as<uint32_t>();
    a.tr_ryr = d_tryr.as<uint32_t>();
    a.tr_cass = d_tcass.p;
    a.tr_cajsr = d_tcajsr.p;
    a.tr_mode = codec ? 1 : 0;
    a.tr_ncru = ncr;
    a.tr_gate = d_gate.as<uint32_t>();
    a.tr_clch = d_clch.as<uint32_t>();
    a.tr_ryrc = d_ryrc.as<uint32_t>();
    a.tr_cass_f = d_cassf.as<float>();
    a.tr_cajsr_f = d_cajsrf.as<float>();
    a.tr_sums = d_sums.as<unsigned long long>();
    CK(c, cudaMemsetAsync(c->d_status.p, 0, sizeof(int) * c->n_cells, c->stream));
    std::vector<unsigned long long> h_sums;
    std::vector<double> h_t, h_glob, h_cur;
    std::vector<uint32_t> h_lcc, h_flags, h_ryr;
    std::vector<unsigned char> h_cass, h_cajsr;
    float total_ms = 0.f;
    int64_t done = 0;
    while (done < n_steps) {
        const int n = (int)std::min<int64_t>(chunk, n_steps - done);
        a.run_step0 = done;
        a.n_steps = n;
        // records of this launch: r in [r_lo, r_hi]
        int64_t r_lo = 0, r_hi = -1;
        if (recording) {
            r_lo = (done + record_every - 1) / record_every;
            r_hi = (done + n - 1) / record_every;
            r_hi = std::min<int64_t>(r_hi, tr->max_records - 1);
            a.rec_base = r_lo;
        }
        if (sums) CK(c, cudaMemsetAsync(d_sums.p, 0, d_sums.n, c->stream));
        CK(c, cudaEventRecord(c->ev0, c->stream));
        const int e = c->precision == GW_PRECISION_FP64 ? launch_engine_fp64(a, c->shape, c->stream, c->ode64)
                                                        : launch_engine_fp32(a, c->shape, c->stream, c->ode64);
        if (e != 0) return fail(c, GW_ERR_CUDA, "engine launch: %s", cudaGetErrorString((cudaError_t)e));
        CK(c, cudaEventRecord(c->ev1, c->stream));
        c->stats.launches++;
        if (recording && r_hi >= r_lo) {
            const int64_t nr = r_hi - r_lo + 1;
            if (currents) {
                const int64_t nt = (int64_t)c->n_cells * nr;
                currents_kernel<<<(unsigned)((nt + 127) / 128), 128, 0, c->stream>>>(
                    c->d_cs.as<CellStatic>(), d_glob.as<double>(), d_sums.as<unsigned long long>(), rec_cap, (int)nr,
                    c->n_cells, d_cur.as<double>());
                CK(c, cudaGetLastError());
            }
            CK(c, cudaStreamSynchronize(c->stream));
            if (currents) {
                h_cur.resize((size_t)GW_CURRENTS * rec_cap * c->n_cells);
                CK(c, cudaMemcpy(h_cur.data(), d_cur.p, d_cur.n, cudaMemcpyDeviceToHost));
                for (int cell = 0; cell < c->n_cells; ++cell)
                    std::memcpy(tr->currents + ((int64_t)cell * tr->max_records + r_lo) * GW_CURRENTS,
                                h_cur.data() + (int64_t)cell * rec_cap * GW_CURRENTS,
                                sizeof(double) * GW_CURRENTS * nr);
            }
            if (tr->cru_sums) {
                h_sums.resize((size_t)kSumFields * rec_cap * c->n_cells);
                CK(c, cudaMemcpy(h_sums.data(), d_sums.p, d_sums.n, cudaMemcpyDeviceToHost));
                for (int cell = 0; cell < c->n_cells; ++cell)
                    for (int64_t r = 0; r < nr; ++r)
                        for (int f = 0; f < kSumFields; ++f) {
                            const long long v = (long long)h_sums[((size_t)cell * rec_cap + r) * kSumFields + f];
                            const bool ca = f == GW_SUM_CASS_CONDUCTING || f == GW_SUM_CASS || f == GW_SUM_CAJSR;
                            tr->cru_sums[((int64_t)cell * tr->max_records + r_lo + r) * kSumFields + f] =
                                ca ? std::ldexp((double)v, -40) : (double)v;
                        }
            }
            if (codec && tr_cell >= 0) {
                const size_t n4 = (size_t)nr * ncr * 4, o4 = (size_t)r_lo * ncr * 4;
                if (tr->LCC_i8) CK(c, cudaMemcpy(tr->LCC_i8 + o4, d_tlcc.p, n4, cudaMemcpyDeviceToHost));
                if (tr->LCC_inactivation_u8)
                    CK(c, cudaMemcpy(tr->LCC_inactivation_u8 + o4, d_gate.p, n4, cudaMemcpyDeviceToHost));
                if (tr->ClCh_u8) CK(c, cudaMemcpy(tr->ClCh_u8 + o4, d_clch.p, n4, cudaMemcpyDeviceToHost));
                if (tr->RyR_i16) CK(c, cudaMemcpy(tr->RyR_i16 + o4, d_ryrc.p, 2 * n4, cudaMemcpyDeviceToHost));
                if (tr->CaSS_f32) CK(c, cudaMemcpy(tr->CaSS_f32 + o4, d_cassf.p, 4 * n4, cudaMemcpyDeviceToHost));
                if (tr->CaJSR_f32)
                    CK(c, cudaMemcpy(tr->CaJSR_f32 + (size_t)r_lo * ncr, d_cajsrf.p, n4, cudaMemcpyDeviceToHost));
            }
            h_t.resize(nr);
            CK(c, cudaMemcpy(h_t.data(), d_t.p, sizeof(double) * nr, cudaMemcpyDeviceToHost));
            if (tr->t)
                for (int64_t r = 0; r < nr; ++r) tr->t[r_lo + r] = h_t[r];
            if (tr->globals) {
                h_glob.resize((size_t)kNumGlobals * rec_cap * c->n_cells);
                CK(c, cudaMemcpy(h_glob.data(), d_glob.p, h_glob.size() * sizeof(double), cudaMemcpyDeviceToHost));
                for (int cell = 0; cell < c->n_cells; ++cell)
                    for (int64_t r = 0; r < nr; ++r)
                        std::memcpy(tr->globals + ((int64_t)cell * tr->max_records + r_lo + r) * kNumGlobals,
                                    h_glob.data() + ((int64_t)cell * rec_cap + r) * kNumGlobals,
                                    sizeof(double) * kNumGlobals);
            }
            if (planes && tr_cell >= 0) {
                h_lcc.resize(stride * nr);
                h_flags.resize(stride * nr);
                h_ryr.resize(6 * stride * nr);
                h_cass.resize(c->rsize * 4 * stride * nr);
                h_cajsr.resize(c->rsize * stride * nr);
                CK(c, cudaMemcpy(h_lcc.data(), d_tlcc.p, 4 * stride * nr, cudaMemcpyDeviceToHost));
                CK(c, cudaMemcpy(h_flags.data(), d_tflags.p, 4 * stride * nr, cudaMemcpyDeviceToHost));
                CK(c, cudaMemcpy(h_ryr.data(), d_tryr.p, 4 * 6 * stride * nr, cudaMemcpyDeviceToHost));
                CK(c, cudaMemcpy(h_cass.data(), d_tcass.p, c->rsize * 4 * stride * nr, cudaMemcpyDeviceToHost));
                CK(c, cudaMemcpy(h_cajsr.data(), d_tcajsr.p, c->rsize * stride * nr, cudaMemcpyDeviceToHost));
                for (int64_t r = 0; r < nr; ++r) {
                    const int64_t R = r_lo + r;
                    for (int i = 0; i < ncr; ++i) {
                        const uint32_t w = h_lcc[r * stride + i], f = h_flags[r * stride + i];
                        for (int j = 0; j < 4; ++j) {
                            const int64_t o = (R * ncr + i) * 4 + j;
                            if (tr->LCC) tr->LCC[o] = (int)((w >> (8 * j)) & 0xFF);
                            if (tr->LCC_inactivation) tr->LCC_inactivation[o] = (int)((f >> j) & 1);
                            if (tr->ClCh) tr->ClCh[o] = (int)((f >> (4 + j)) & 1);
                            if (tr->RyR)
                                for (int k = 0; k < 6; ++k)
                                    tr->RyR[o * 6 + k] = (int)(int8_t)((h_ryr[(r * 6 + k) * stride + i] >> (8 * j)) & 0xFF);
                            if (tr->CaSS) {
                                const int64_t src = (r * 4 + j) * stride + i;
                                tr->CaSS[o] = c->rsize == 8 ? reinterpret_cast<double *>(h_cass.data())[src]
                                                            : (double)reinterpret_cast<float *>(h_cass.data())[src];
                            }
                        }
                        if (tr->CaJSR) {
                            const int64_t src = r * stride + i;
                            tr->CaJSR[R * ncr + i] = c->rsize == 8 ? reinterpret_cast<double *>(h_cajsr.data())[src]
                                                                   : (double)reinterpret_cast<float *>(h_cajsr.data())[src];
                        }
                    }
                }
            }
            tr->n_written = std::max<int64_t>(tr->n_written, r_hi + 1);
        }
        CK(c, cudaEventSynchronize(c->ev1));
        float ms = 0.f;
        CK(c, cudaEventElapsedTime(&ms, c->ev0, c->ev1));
        total_ms += ms;
        done += n;
    }
    CK(c, cudaStreamSynchronize(c->stream));
    CK(c, cudaGetLastError());
    c->stats.kernel_ms += total_ms;
    c->stats.steps += (uint64_t)n_steps;
    unsigned long long ev = 0;
    CK(c, cudaMemcpy(&ev, c->d_events.p, sizeof ev, cudaMemcpyDeviceToHost));
    c->stats.events = ev;
    std::vector<int> st(c->n_cells);
    CK(c, cudaMemcpy(st.data(), c->d_status.p, sizeof(int) * c->n_cells, cudaMemcpyDeviceToHost));
    for (int i = 0; i < c->n_cells; ++i)
        if (st[i] != 0) {
            const char *what = st[i] == GW_ERR_EVENT_CAP ? "a CRU exceeded the per-step jump cap"
                               : st[i] == GW_ERR_NERNST  ? "non-positive concentration in a Nernst potential"
                               : st[i] == GW_ERR_NONFINITE ? "a global state variable became NaN/Inf"
                               : st[i] == GW_ERR_SYNC_TIMEOUT ? "a bounded wait in the engine kernel ran out"
                                                           : "error";
            return fail(c, st[i], "cell %d: %s", i, what);
        }
    return GW_OK;
}

int gw_run_noalloc(gw_ctx *c, double dt, int64_t n_steps, int record_every, gw_trace *tr) {
    if (!c) return GW_ERR_INVALID_ARGUMENT;
    if (!(dt > 0.0) || !std::isfinite(dt)) return fail(c, GW_ERR_INVALID_ARGUMENT, "dt must be > 0");
    if (n_steps < 0) return fail(c, GW_ERR_INVALID_ARGUMENT, "n_steps must be >= 0");
    if (record_every < 0) return fail(c, GW_ERR_INVALID_ARGUMENT, "record_every must be >= 0");
    CK(c, cudaSetDevice(c->device));
    if (tr) tr->n_written = 0;
    const bool recording = tr && record_every > 0 && tr->max_records > 0;
    if (recording && (tr->cru_sums || tr->LCC_i8 || tr->LCC_inactivation_u8 || tr->ClCh_u8 || tr->RyR_i16 ||
                      tr->CaSS_f32 || tr->CaJSR_f32 || tr->currents))
        return fail(c, GW_ERR_INVALID_ARGUMENT, "gw_run_noalloc records the int32/double trace arrays only");
    const bool cru_fields = recording && (tr->CaSS || tr->CaJSR || tr->LCC || tr->LCC_inactivation || tr->RyR || tr->ClCh);
    const int tr_cell = cru_fields ? tr->cru_cell : -1;
    if (tr_cell >= c->n_cells) return fail(c, GW_ERR_INVALID_ARGUMENT, "trace cell out of range");
    {
        int rc = pull_dyn(c);
        if (rc) return rc;
        for (int i = 0; i < c->n_cells; ++i)
            if (c->dyn_host[i].step + (uint64_t)n_steps > 0xFFFFFFFFull)
                return fail(c, GW_ERR_INVALID_ARGUMENT, "more than 2^32 steps in one context");
    }
    unsigned char *scratch = nullptr;
    {
        int rc = noalloc_scratch(c, &scratch);
        if (rc) return rc;
    }
    // Scratch bytes of one record (engine planes + reference layouts), 256-byte padding included.
    const int ncr = tr_cell >= 0 ? c->ncru[tr_cell] : 0;
    const int64_t stride = tr_cell >= 0 ? ((int64_t)ncr + 31) / 32 * 32 : 0;
    auto pad = [](size_t b) { return (b + 255) & ~(size_t)255; };
    auto bytes_for = [&](int64_t nrec) -> size_t {
        if (!recording) return 0;
        size_t b = pad(sizeof(double) * nrec) + pad(sizeof(double) * kNumGlobals * nrec * c->n_cells);
        if (tr_cell >= 0) {
            b += 2 * pad(4 * stride * nrec) + pad(4 * 6 * stride * nrec) + pad(c->rsize * 4 * stride * nrec) +
                 pad(c->rsize * stride * nrec);
            const size_t n4 = (size_t)nrec * ncr * 4;
            if (tr->LCC) b += pad(4 * n4);
            if (tr->LCC_inactivation) b += pad(4 * n4);
            if (tr->ClCh) b += pad(4 * n4);
            if (tr->RyR) b += pad(4 * 6 * n4);
            if (tr->CaSS) b += pad(8 * n4);
            if (tr->CaJSR) b += pad(8 * (size_t)nrec * ncr);
        }
        return b;
    };
    // Steps per launch: the engine's launch length, shortened so that its records fit the scratch.
    int64_t chunk = c->steps_per_launch;
    int64_t rec_cap = 0;
    if (recording) {
        if (bytes_for(3) > kNoallocScratchBytes) {
            if (tr_cell < 0)
                return fail(c, GW_ERR_INVALID_ARGUMENT,
                            "a trace record of the globals of %d cells needs about %zu bytes of staging and "
                            "gw_run_noalloc stages at least 3 records in its %zu-byte scratch; split the cells "
                            "over several contexts or use gw_run",
                            c->n_cells, bytes_for(1), kNoallocScratchBytes);
            return fail(c, GW_ERR_INVALID_ARGUMENT,
                        "a trace record of this context needs about %zu bytes of staging and gw_run_noalloc stages at "
                        "least 3 records in its %zu-byte scratch; record fewer CRU fields or use gw_run",
                        bytes_for(1), kNoallocScratchBytes);
        }
        while (bytes_for(chunk / record_every + 2) > kNoallocScratchBytes) chunk = std::max<int64_t>(1, chunk / 2);
        rec_cap = std::min<int64_t>(tr->max_records, chunk / record_every + 2);
    }
    ScratchCursor sc{scratch, 0};
    KernelArgs a = base_args(c);
    a.dt = dt;
    a.record_every = recording ? record_every : 0;
    a.rec_cap = (int)rec_cap;
    a.tr_cell = tr_cell;
    a.tr_cru_stride = stride;
    int32_t *u_lcc = nullptr, *u_lcci = nullptr, *u_clch = nullptr, *u_ryr = nullptr;
    double *u_cass = nullptr, *u_cajsr = nullptr;
    if (recording) {
        a.tr_t = sc.take<double>(sizeof(double) * rec_cap);
        a.tr_glob = sc.take<double>(sizeof(double) * kNumGlobals * rec_cap * c->n_cells);
        if (tr_cell >= 0) {
            a.tr_lcc = sc.take<uint32_t>(4 * stride * rec_cap);
            a.tr_flags = sc.take<uint32_t>(4 * stride * rec_cap);
            a.tr_ryr = sc.take<uint32_t>(4 * 6 * stride * rec_cap);
            a.tr_cass = sc.take<unsigned char>(c->rsize * 4 * stride * rec_cap);
            a.tr_cajsr = sc.take<unsigned char>(c->rsize * stride * rec_cap);
            const size_t n4 = (size_t)rec_cap * ncr * 4;
            if (tr->LCC) u_lcc = sc.take<int32_t>(4 * n4);
            if (tr->LCC_inactivation) u_lcci = sc.take<int32_t>(4 * n4);
            if (tr->ClCh) u_clch = sc.take<int32_t>(4 * n4);
            if (tr->RyR) u_ryr = sc.take<int32_t>(4 * 6 * n4);
            if (tr->CaSS) u_cass = sc.take<double>(8 * n4);
            if (tr->CaJSR) u_cajsr = sc.take<double>(8 * (size_t)rec_cap * ncr);
        }
    }
    if (sc.used > kNoallocScratchBytes) return fail(c, GW_ERR_INVALID_ARGUMENT, "trace staging exceeds the scratch");
    CK(c, cudaMemsetAsync(c->d_status.p, 0, sizeof(int) * c->n_cells, c->stream));
    float total_ms = 0.f;
    int64_t done = 0;
    while (done < n_steps) {
        const int n = (int)std::min<int64_t>(chunk, n_steps - done);
        a.run_step0 = done;
        a.n_steps = n;
        int64_t r_lo = 0, r_hi = -1;
        if (recording) {
            r_lo = (done + record_every - 1) / record_every;
            r_hi = std::min<int64_t>((done + n - 1) / record_every, tr->max_records - 1);
            a.rec_base = r_lo;
        }
        CK(c, cudaEventRecord(c->ev0, c->stream));
        const int e = c->precision == GW_PRECISION_FP64 ? launch_engine_fp64(a, c->shape, c->stream, c->ode64)
                                                        : launch_engine_fp32(a, c->shape, c->stream, c->ode64);
        if (e != 0) return fail(c, GW_ERR_CUDA, "engine launch: %s", cudaGetErrorString((cudaError_t)e));
        CK(c, cudaEventRecord(c->ev1, c->stream));
        c->stats.launches++;
        if (recording && r_hi >= r_lo) {
            const int64_t nr = r_hi - r_lo + 1;
            if (tr->t)
                CK(c, cudaMemcpyAsync(tr->t + r_lo, a.tr_t, sizeof(double) * nr, cudaMemcpyDeviceToHost, c->stream));
            if (tr->globals)
                CK(c, cudaMemcpy2DAsync(tr->globals + r_lo * kNumGlobals, sizeof(double) * kNumGlobals * tr->max_records,
                                        a.tr_glob, sizeof(double) * kNumGlobals * rec_cap,
                                        sizeof(double) * kNumGlobals * nr, c->n_cells, cudaMemcpyDeviceToHost, c->stream));
            if (tr_cell >= 0 && ncr > 0) {
                const int64_t total = nr * ncr;
                const int threads = 256;
                const unsigned blocks = (unsigned)((total + threads - 1) / threads);
                unpack_trace_kernel<<<blocks, threads, 0, c->stream>>>(
                    (int)nr, ncr, stride, c->rsize == 8, a.tr_lcc, a.tr_flags, a.tr_ryr, a.tr_cass, a.tr_cajsr, u_lcc,
                    u_lcci, u_clch, u_ryr, u_cass, u_cajsr);
                CK(c, cudaGetLastError());
                const size_t n4 = (size_t)nr * ncr * 4;
                const int64_t o4 = r_lo * ncr * 4;
                if (tr->LCC) CK(c, cudaMemcpyAsync(tr->LCC + o4, u_lcc, 4 * n4, cudaMemcpyDeviceToHost, c->stream));
                if (tr->LCC_inactivation)
                    CK(c, cudaMemcpyAsync(tr->LCC_inactivation + o4, u_lcci, 4 * n4, cudaMemcpyDeviceToHost, c->stream));
                if (tr->ClCh) CK(c, cudaMemcpyAsync(tr->ClCh + o4, u_clch, 4 * n4, cudaMemcpyDeviceToHost, c->stream));
                if (tr->RyR) CK(c, cudaMemcpyAsync(tr->RyR + o4 * 6, u_ryr, 4 * 6 * n4, cudaMemcpyDeviceToHost, c->stream));
                if (tr->CaSS) CK(c, cudaMemcpyAsync(tr->CaSS + o4, u_cass, 8 * n4, cudaMemcpyDeviceToHost, c->stream));
                if (tr->CaJSR)
                    CK(c, cudaMemcpyAsync(tr->CaJSR + r_lo * ncr, u_cajsr, 8 * (size_t)nr * ncr, cudaMemcpyDeviceToHost, c->stream));
            }
            // the next launch reuses the staging area
            CK(c, cudaStreamSynchronize(c->stream));
            tr->n_written = std::max<int64_t>(tr->n_written, r_hi + 1);
        }
        CK(c, cudaEventSynchronize(c->ev1));
        float ms = 0.f;
        CK(c, cudaEventElapsedTime(&ms, c->ev0, c->ev1));
        total_ms += ms;
        done += n;
    }
    CK(c, cudaStreamSynchronize(c->stream));
    CK(c, cudaGetLastError());
    c->stats.kernel_ms += total_ms;
    c->stats.steps += (uint64_t)n_steps;
    unsigned long long ev = 0;
    CK(c, cudaMemcpy(&ev, c->d_events.p, sizeof ev, cudaMemcpyDeviceToHost));
    c->stats.events = ev;
    int st[64];
    for (int i0 = 0; i0 < c->n_cells; i0 += 64) {
        const int nb = std::min(64, c->n_cells - i0);
        CK(c, cudaMemcpy(st, c->d_status.as<int>() + i0, sizeof(int) * nb, cudaMemcpyDeviceToHost));
        for (int i = 0; i < nb; ++i)
            if (st[i] != 0) {
                const char *what = st[i] == GW_ERR_EVENT_CAP ? "a CRU exceeded the per-step jump cap"
                                   : st[i] == GW_ERR_NERNST  ? "non-positive concentration in a Nernst potential"
                                   : st[i] == GW_ERR_NONFINITE ? "a global state variable became NaN/Inf"
                                   : st[i] == GW_ERR_SYNC_TIMEOUT ? "a bounded wait in the engine kernel ran out"
                                                               : "error";
                return fail(c, st[i], "cell %d: %s", i0 + i, what);
            }
    }
    return GW_OK;
}

int gw_math_check(const double *x, int64_t n, double *exp_out, double *log_out) {
    if (!x || !exp_out || !log_out || n < 0 || n > (int64_t)1 << 26)
        return fail(nullptr, GW_ERR_INVALID_ARGUMENT, "bad arguments to gw_math_check");
    if (n == 0) return GW_OK;
    DevBuf dx, de, dl;
    gw_ctx *c = nullptr;
    CK(c, dx.alloc(sizeof(double) * n));
    CK(c, de.alloc(sizeof(double) * n));
    CK(c, dl.alloc(sizeof(double) * n));
    CK(c, cudaMemcpy(dx.p, x, sizeof(double) * n, cudaMemcpyHostToDevice));
    const int e = math_check_dev(dx.as<double>(), (int)n, de.as<double>(), dl.as<double>());
    if (e != 0) return fail(nullptr, GW_ERR_CUDA, "math check launch: %s", cudaGetErrorString((cudaError_t)e));
    CK(c, cudaMemcpy(exp_out, de.p, sizeof(double) * n, cudaMemcpyDeviceToHost));
    CK(c, cudaMemcpy(log_out, dl.p, sizeof(double) * n, cudaMemcpyDeviceToHost));
    return GW_OK;
}

int gw_screen_check(const gw_params *p, int nCRU, int64_t n, const uint32_t *chan, const double *cass,
                    const double *sv, const double *t, const double *dt, uint64_t seed, int32_t *out,
                    double *jump) {
    if (!p || nCRU < 1 || !chan || !cass || !sv || !t || !dt || !out || !jump || n < 0 || n > (int64_t)1 << 24)
        return fail(nullptr, GW_ERR_INVALID_ARGUMENT, "bad arguments to gw_screen_check");
    if (n == 0) return GW_OK;
    CellStatic C;
    make_cell_static(*p, nCRU, C);
    DevBuf dc, dch, dx, ds, dtt, ddt, dout, dj;
    gw_ctx *c = nullptr;
    CK(c, dc.alloc(sizeof(CellStatic)));
    CK(c, dch.alloc(sizeof(uint32_t) * 8 * n));
    CK(c, dx.alloc(sizeof(double) * 4 * n));
    CK(c, ds.alloc(sizeof(double) * kSvCount * n));
    CK(c, dtt.alloc(sizeof(double) * n));
    CK(c, ddt.alloc(sizeof(double) * n));
    CK(c, dout.alloc(sizeof(int32_t) * 2 * n));
    CK(c, dj.alloc(sizeof(double) * n));
    CK(c, cudaMemcpy(dc.p, &C, sizeof(CellStatic), cudaMemcpyHostToDevice));
    CK(c, cudaMemcpy(dch.p, chan, sizeof(uint32_t) * 8 * n, cudaMemcpyHostToDevice));
    CK(c, cudaMemcpy(dx.p, cass, sizeof(double) * 4 * n, cudaMemcpyHostToDevice));
    CK(c, cudaMemcpy(ds.p, sv, sizeof(double) * kSvCount * n, cudaMemcpyHostToDevice));
    CK(c, cudaMemcpy(dtt.p, t, sizeof(double) * n, cudaMemcpyHostToDevice));
    CK(c, cudaMemcpy(ddt.p, dt, sizeof(double) * n, cudaMemcpyHostToDevice));
    const int e = screen_check_dev(static_cast<const CellStatic *>(dc.p), (int)n, static_cast<const uint32_t *>(dch.p),
                                   dx.as<double>(), ds.as<double>(), dtt.as<double>(), ddt.as<double>(), seed,
                                   static_cast<int *>(dout.p), dj.as<double>());
    if (e != 0) return fail(nullptr, GW_ERR_CUDA, "screen check launch: %s", cudaGetErrorString((cudaError_t)e));
    CK(c, cudaMemcpy(out, dout.p, sizeof(int32_t) * 2 * n, cudaMemcpyDeviceToHost));
    CK(c, cudaMemcpy(jump, dj.p, sizeof(double) * n, cudaMemcpyDeviceToHost));
    return GW_OK;
}

int gw_get_time(gw_ctx *c, int cell, double *t, uint64_t *step) {
    int rc = check_cell(c, cell);
    if (rc) return rc;
    cudaSetDevice(c->device);
    if ((rc = pull_dyn(c))) return rc;
    if (t) *t = c->dyn_host[cell].t;
    if (step) *step = c->dyn_host[cell].step;
    return GW_OK;
}

int gw_set_time(gw_ctx *c, int cell, double t, uint64_t step) {
    int rc = check_cell(c, cell);
    if (rc) return rc;
    if (!std::isfinite(t) || step > 0xFFFFFFFFull) return fail(c, GW_ERR_INVALID_ARGUMENT, "bad time or step");
    cudaSetDevice(c->device);
    if ((rc = pull_dyn(c))) return rc;
    c->dyn_host[cell].t = t;
    c->dyn_host[cell].step = step;
    return push_dyn(c);
}

int gw_get_stats(gw_ctx *c, gw_stats *s) {
    if (!c || !s) return GW_ERR_INVALID_ARGUMENT;
    *s = c->stats;
    s->device_allocs = g_device_allocs.load(std::memory_order_relaxed);
    return GW_OK;
}

int gw_last_error(gw_ctx *c, char *msg, size_t len) {
    if (!msg || len == 0) return GW_ERR_INVALID_ARGUMENT;
    const std::string &e = c ? c->err : g_create_error;
    std::snprintf(msg, len, "%s", e.c_str());
    return GW_OK;
}

int gw_global_step_host(const gw_params *p, int nCRU, double *g, const double *sums, double Istim,
                        double dt, double *sv) {
    if (!p || nCRU <= 0 || !g || !sums) return fail(nullptr, GW_ERR_INVALID_ARGUMENT, "bad arguments");
    CellStatic cs;
    make_cell_static(*p, nCRU, cs);
    static thread_local OdeProgram prog;
    static thread_local double consts[kOdeMaxConsts];
    const bool fast = p->Hf == 0.75 && p->Hr == 0.75;
    if (!ode_program_build(cs, fast, &prog, consts)) return fail(nullptr, GW_ERR_UNSUPPORTED, "ODE program too large");
    double tmp[kSvCount];
    ode_program_step_host(prog, consts, g, sums, Istim, dt, sv ? sv : tmp);
    return GW_OK;
}

int gw_simulate(const gw_params *p, int nCRU, double step_size, int64_t num_steps,
                const double *Istim, int record_every, const double *init_CaSS,
                const double *init_CaJSR, const int32_t *init_LCC,
                const int32_t *init_LCC_inactivation, const int32_t *init_RyR,
                const int32_t *init_ClCh, const gw_globals *init_globals, const char *prng,
                uint64_t seed, int precision, gw_trace *trace) {
    static const char *kEngines[] = {"mt19937",       "mt19937_64",    "xoshiro256+",
                                     "xoshiro256++",  "xoshiro256**",  "xoroshiro128+",
                                     "xoroshiro128++", "xoroshiro128**"};
    bool ok = false;
    for (const char *e : kEngines)
        if (prng && std::strcmp(prng, e) == 0) ok = true;
    if (!ok) return fail(nullptr, GW_ERR_INVALID_ARGUMENT, "%s", prng ? prng : "(null)");
    if (!p || nCRU <= 0 || num_steps < 0 || record_every <= 0 || !init_globals)
        return fail(nullptr, GW_ERR_INVALID_ARGUMENT, "bad arguments to gw_simulate");
    gw_ensemble_desc d;
    std::memset(&d, 0, sizeof d);
    int32_t n = nCRU;
    d.n_cells = 1;
    d.ncru = &n;
    d.params = p;
    d.precision = precision;
    d.seed = seed;
    d.device = 0;
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess) d.device = dev;
    gw_ctx *c = nullptr;
    int rc = gw_create(&d, &c);
    if (rc) return rc;
    rc = gw_set_globals(c, 0, init_globals);
    if (!rc) rc = gw_set_crus(c, 0, init_CaSS, init_CaJSR, init_LCC, init_LCC_inactivation, init_RyR, init_ClCh, nullptr);
    if (!rc) rc = gw_set_stimulus_samples(c, 0, Istim, Istim ? num_steps : 0);
    if (!rc) rc = gw_run(c, step_size, num_steps, record_every, trace);
    if (rc) g_create_error = c->err;
    gw_destroy(c);
    return rc;
}

}  // extern "C"
