"""Benchmark: CRU-steps/s and simulated ms per wall-second of the Greenstein-Winslow hybrid SSA,
batched GPU vs plain GPU vs the reference's CPU path.

Workload of the JSON line's `value` (one GPU): one full cell of 12,500 CRUs (NCaRU = 12,500, so
each simulated CRU stands for one real CRU), reference default parameters, GW::GlobalState resting
globals, the reference's random initial CRU distributions, dt = 1e-3 ms, 1 Hz pacing with a
+100 pA/pF, 0.5 ms stimulus (the reference integrates dV = dt (Istim - sum I), so the usual
-100 pA/pF inward stimulus is +100 here).  CRU state FP32, global ODE FP64 with compensated flux
reduction.  Synthetic seeded input.

Timed window: one whole beat.  The K timed steps are K consecutive windows of 1000/K ms that cover
0-1000 ms of the beat (upstroke, Ca release, plateau, repolarisation, rest); the W warm-up steps
run the same windows first on the same context, which is then restored to its t = 0 checkpoint.
Between timed steps a 256 MB buffer is written (L2 flush; the cell's 0.9 MB state would otherwise
stay in L2 between launches).

  value        CRU-steps/s over the beat, state resident on the device, CUDA events on the
               engine's stream around every engine launch
  e2e          the same beat through the reference-facing C ABI (gw_simulate: host arrays in, the
               per-step stimulus samples uploaded, the last step's state copied back and passed to
               the next call, a fresh context per call, as chained run() calls of the reference)
  paths        plain GPU (the same cell, one launch and one host synchronisation per global step,
               sampled at every window start of the beat), batched GPU (256 cells of 2,000-12,500
               CRUs, log-normal per-cell parameters and 400-1000 ms cycle lengths, one launch,
               0-400 ms of every cell's beat), config 5 (1,024 x 12,500 CRUs, 2 Hz, cells spread over
               16 phases of the beat from a one-beat phase library, timed over one 31.25 ms stratum
               so that the whole beat is covered once), and config 1 (one 1,250-CRU cell, FP64
               throughout, 500 ms) on the GPU
               beside the CPU port running the same config in full
  roofline     the engine kernel against HBM (algorithmic bytes = the 72-byte FP32 CRU state read
               and written once per CRU-step); issue_roofline: warp instructions issued against
               the issue rate of the SMs the cell uses (what binds a single cell)
  accuracy     the FP32 path's error against the FP64 oracle at the headline config with common
               random numbers (1 and 200 steps from the same 12,500-CRU state at four points of
               the beat), and FP32 vs FP64 ensemble statistics (64 cells x 500 CRUs, 450 ms)
  cpu_baseline the oracle port of the reference's C++ built with the reference's Release flags,
               OpenMP over CRUs on all host cores, timed on the same beat phases: a 1,250-CRU cell
               runs the beat on the CPU, its state at each window start is tiled to 12,500 CRUs,
               and a bounded sample is timed from each

--impl reference times that CPU implementation alone (the oracle port; the reference's own C++
cannot be built on the GPU host, which has no copy of its sources).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(REPO, "gw-model_gb300"), os.path.join(REPO, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

NCRU = 12500
DT = 1e-3
PERIOD = 1000.0
STIM_AMP, STIM_DUR = 100.0, 0.5
METRIC = "CRU-steps/s and sim-ms/wall-s: batched vs plain GPU vs CPU, at KS/FP64 tol"
# FP32 CRU state per CRU: LCC states 4 B, gate + ClCh bits 4 B, RyR counts 24 B, CaSS 16 B,
# JLCC 16 B, CaJSR 4 B, CaJSR compensation 4 B = 72 B, read and written once per CRU-step.
BYTES_PER_CRU_STEP = 2 * 72
# From the ncu captures of the engine kernel on this workload (profiles/engine_kernel_cell12500.txt
# and profiles/engine_kernel_cell12500_instmix.txt, the launch at 0-1 ms of the beat): DRAM bytes
# (read + write) of one 1000-step launch, and warp instructions issued per CRU-step.
TRAFFIC_PER_LAUNCH = 1.05472e6
WARP_INST_PER_CRU_STEP = 31.25
# The same for config 3's ensemble kernel (profiles/engine_kernel_batched256.txt, one 100-step launch
# at 20 ms): DRAM bytes per launch and CRU, and warp instructions per CRU-step.
BATCHED_TRAFFIC_PER_LAUNCH_CRU = 213.9e6 / 1870540
BATCHED_WARP_INST_PER_CRU_STEP = 38.8
CPU_PRE_NCRU = 1250   # the CPU's beat run, tiled x10 to 12,500 CRUs at each window start


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--beat-ms", type=float, default=PERIOD, help="simulated time the K timed steps cover")
    ap.add_argument("--cells", type=int, default=1, help="cells of the headline configuration per GPU")
    ap.add_argument("--no-extras", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=10.0, help="CPU time of the timed samples")
    ap.add_argument("--config4", type=float, default=0.0, metavar="MS",
                    help="only run config 4 (32 cells x 5,000 CRUs, adjoint of a V-trace MSE) over MS ms after "
                         "one stimulus and print its timing as one JSON line")
    ap.add_argument("--config4-cells", type=int, default=32)
    ap.add_argument("--config4-checkpoint", type=int, default=200, help="global steps between adjoint checkpoints")
    ap.add_argument("--profile-batched", type=int, default=0, metavar="LAUNCHES",
                    help="only run config 3's ensemble with 100 steps per launch: 200 launches (0-20 ms), then "
                         "LAUNCHES more (the launches an ncu capture takes)")
    ap.add_argument("--ks-full-cells", type=float, default=0.0, metavar="MS",
                    help="only run the FP32 vs FP64 KS comparison of 200 replicate 12,500-CRU cells over the "
                         "first MS ms after a stimulus and print it as one JSON line")
    ap.add_argument("--config5-accuracy", type=int, default=0, metavar="BEATS",
                    help="only run config 5's FP32 vs FP64 APD90 / peak-Cai comparison over BEATS beats at 2 Hz "
                         "(64 cells) and print it as one JSON line")
    return ap.parse_args()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True,
                                     timeout=5).stdout.strip()
                if out:
                    self.samples.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4)
                          if len(s) > 3 + i and s[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


class L2Flush:
    """Writes a 256 MB device buffer (twice the 129 MB L2) between timed steps."""

    def __init__(self, device):
        self.buf = None
        try:
            import torch

            if torch.cuda.is_available():
                self.buf = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{device}")
                self.torch = torch
        except Exception:
            self.buf = None

    def __call__(self, k=0):
        if self.buf is not None:
            self.buf.fill_(k & 0xFF)
            self.torch.cuda.synchronize(self.buf.device)

    def note(self):
        return "256 MB buffer written between timed steps (L2 flush)" if self.buf is not None else \
            "no L2 flush (torch CUDA unavailable)"


def peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def pulse(t: float) -> float:
    """The 1 Hz stimulus at time t, the engine's pulse-train formula."""
    tb = t - PERIOD * float(int(t / PERIOD))
    return STIM_AMP if tb < STIM_DUR else 0.0


def window_steps(K: int, beat_ms: float) -> int:
    return max(1, int(round(beat_ms / K / DT)))


# ---------------------------------------------------------------------------------------------
# CPU: the oracle port of the reference (Release flags), timed at matching beat phases
# ---------------------------------------------------------------------------------------------

def cpu_phase_states(K: int, span: int, threads: int):
    """A 1,250-CRU cell (NCaRU 12,500) through K windows of `span` steps on the CPU; its state (globals,
    CRU arrays, per-CRU fluxes) at each window start."""
    import pyoracle as po

    po.build()
    po.timed_lib().orc_set_threads(threads)
    p = po.default_params()
    m = po.Model(p, CPU_PRE_NCRU, seed=0, timed=True)
    m.sample_initial_crus()
    m.set_globals(po.default_globals(py=False))
    states = []
    t = 0.0
    for k in range(K):
        states.append((m.globals(), m.crus(), m.fluxes(), t, k * span))
        for _ in range(span):
            m.euler_step(DT, pulse(t))
            t += DT
    return states


def cpu_window_sample(state, steps: int, threads: int, seed: int):
    """Times `steps` steps of a 12,500-CRU cell (the state tiled x10) on the CPU; returns seconds."""
    import numpy as np

    import pyoracle as po

    g, s, (JLCC, Jxfer, Jtr), t, step = state
    f = NCRU // CPU_PRE_NCRU
    tile = po.CRUArrays(NCRU)
    for k in ("CaSS", "CaJSR", "LCC", "LCC_inactivation", "RyR", "ClCh"):
        setattr(tile, k, np.concatenate([getattr(s, k)] * f))
    po.timed_lib().orc_set_threads(threads)
    m = po.Model(po.default_params(), NCRU, seed=seed, timed=True)
    m.set_globals(g)
    m.set_crus(tile)
    # per-CRU fluxes tiled as they are: the global step scales their sum by CRU_factor, which is
    # 10 for the 1,250-CRU run and 1 here, so the sums the global step sees are the same
    m.set_fluxes(np.concatenate([JLCC] * f), np.concatenate([Jxfer] * f), np.concatenate([Jtr] * f))
    m.set_step(step)
    t0 = time.perf_counter()
    for _ in range(steps):
        m.euler_step(DT, pulse(t))
        t += DT
    return time.perf_counter() - t0


def cpu_baseline(K: int, span: int, seconds: float, warmup: int = 0):
    """Whole-beat CPU rate: K samples, one per window start, each ~seconds/K of CPU work."""
    threads = os.cpu_count() or 1
    states = cpu_phase_states(K, span, threads)
    per = max(50, int(seconds / K * 5e7 / NCRU))   # ~seconds/K each at ~5e7 CRU-steps/s
    for w in range(warmup):
        cpu_window_sample(states[w % K], per, threads, seed=900 + w)
    times = [cpu_window_sample(states[k], per, threads, seed=k) for k in range(K)]
    total = sum(times)
    rate = NCRU * per * K / total
    return {"value": rate, "unit": "CRU-steps/s", "cores": threads, "kind": "port",
            "build": "oracle/_build/liboracle_timed.so (-Ofast -funroll-loops, OpenMP over CRUs)",
            "sample": f"{K} samples of {per} steps x {NCRU} CRUs, one at each {span * DT:g} ms window start of "
                      f"the 1 Hz beat (0-{K * span * DT:g} ms; states from a {CPU_PRE_NCRU}-CRU CPU run of the "
                      f"beat tiled x{NCRU // CPU_PRE_NCRU}), {total:.1f} s",
            "per_window_cru_steps_per_s": [NCRU * per / x for x in times]}


def workload_config(args, world=1, K=None, flush_note=None):
    cells = max(args.cells, 1)
    K = K or args.steps
    span = window_steps(K, args.beat_ms)
    return {"workload": f"{'single cell' if cells == 1 else f'{cells} cells'} of {NCRU} CRUs per GPU, "
                        f"1 Hz pacing (+{STIM_AMP:g} pA/pF, {STIM_DUR:g} ms), dt 1e-3 ms, "
                        f"FP32 CRU state, FP64 global ODE",
            "ncru": NCRU, "cells_per_gpu": cells, "window_ms_per_step": span * DT,
            "timed_span_ms": f"0-{K * span * DT:g} of the beat (warm-up on the same windows, then the t = 0 "
                             "state restored)",
            "parallelism": (f"{cells * world} cells partitioned over {world} ranks (contiguous shares, streams "
                            "keyed on the global cell index, no collective on the data path)" if world > 1
                            else "1 GPU"),
            "l2": flush_note or "256 MB buffer written between timed steps (L2 flush)"}


def run_reference(args):
    from gwgb300 import dist as gd

    rank, _, world = gd.env_rank()
    if rank != 0:
        return 0
    K, W = args.steps, args.warmup
    span = window_steps(K, args.beat_ms)
    cb = cpu_baseline(K, span, args.cpu_seconds, warmup=W)
    v = cb["value"]
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "CRU-steps/s",
            "n_gpus": args.gpus, "steps": K, "warmup": W, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(args, world, K, "CPU run; no GPU"),
            "cpu_baseline": cb,
            "e2e": {"value": v, "unit": "CRU-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------------------------

def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.config4:
        print(json.dumps({"config4": config4_measure(0, args.config4, args.config4_cells,
                                                     checkpoint_every=args.config4_checkpoint)}), flush=True)
        return 0
    if args.profile_batched:
        profile_batched(0, args.profile_batched)
        return 0
    if args.ks_full_cells:
        print(json.dumps({"ks_full_cells": ks_full_cells(0, t_ms=args.ks_full_cells)}), flush=True)
        return 0
    if args.config5_accuracy:
        print(json.dumps({"config5_accuracy": config5_accuracy(0, beats=args.config5_accuracy)}), flush=True)
        return 0
    from gwgb300 import Ensemble
    from gwgb300 import dist as gd

    rank, local_rank, world = gd.env_rank()
    d = gd.init()
    K, W = args.steps, max(args.warmup, 3)
    span = window_steps(K, args.beat_ms)
    cells = max(args.cells, 1)
    # one ensemble of cells x world cells, split into contiguous shares (rank r holds global cells
    # r*cells ..), each keyed on its global cell index: the union is the 1-GPU run of all cells
    e = Ensemble.partitioned([NCRU] * (cells * world), world=world, rank=rank, precision="fp32", seed=1000,
                             device=local_rank)
    for c in range(cells):
        e.sample_initial_crus(c)
    e.set_pulse(0.0, PERIOD, STIM_DUR, STIM_AMP)
    ck0 = [e.checkpoint(c) for c in range(cells)]
    for _ in range(W):
        e.run(DT, span)
    for c in range(cells):
        e.restore(c, ck0[c])
    flush = L2Flush(local_rank)
    windows = []       # window-start checkpoints of cell 0 (plain path, accuracy)
    per_step = []
    gd.barrier(d)
    st0 = e.stats()
    t0 = time.perf_counter()
    with ClockSampler(local_rank) as clk:
        for k in range(K):
            if rank == 0 and not args.no_extras:
                windows.append(e.checkpoint(0))
            flush(k)
            a = e.stats()
            e.run(DT, span)
            b = e.stats()
            per_step.append(b["kernel_ms"] - a["kernel_ms"])
    wall = time.perf_counter() - t0
    st1 = e.stats()
    kernel_s = sum(per_step) / 1e3
    kernel_s = gd.max_over_ranks(d, kernel_s)
    wall = gd.max_over_ranks(d, wall)
    cru_steps = NCRU * cells * span * K * world
    value = cru_steps / kernel_s
    launches = int(st1["launches"] - st0["launches"])
    pk, pk_kind = peaks()
    per_launch_steps = span * K / max(launches, 1)
    achieved_gbs = BYTES_PER_CRU_STEP * NCRU * cells * span * K / kernel_s / 1e9
    clocks = clk.summary()
    sm_hz = (clocks.get("sm_mhz") or pk.get("sm_max_mhz", 2070.0)) * 1e6
    sms_used = st1["cluster_ctas"] * (st1["n_clusters"])
    warp_rate = WARP_INST_PER_CRU_STEP * value / world
    line = {"metric": METRIC, "value": value, "unit": "CRU-steps/s", "n_gpus": world,
            "steps": K, "warmup": W, "ms_per_step": kernel_s / K * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(args, world, K, flush.note()),
            "launch_shape": {k: st1[k] for k in ("cluster_ctas", "cta_crus", "threads_per_cta", "n_clusters")},
            "sim_ms_per_wall_s": cells * world * span * K * DT / kernel_s,
            "events_per_cru_step": (st1["events"] - st0["events"]) / max(NCRU * cells * span * K, 1),
            "per_window_us_per_step": [ms * 1e3 / span for ms in per_step],
            "gpu_launches": launches,
            "roofline": {"bound": "hbm", "achieved": achieved_gbs, "peak": pk["hbm_gbs"], "unit": "GB/s",
                         "frac": achieved_gbs / pk["hbm_gbs"],
                         "traffic": TRAFFIC_PER_LAUNCH if per_launch_steps == 1000 and cells == 1 else None,
                         "traffic_unit": "bytes per launch (ncu dram read + write)",
                         "peak_kind": pk_kind, "bytes_per_cru_step": BYTES_PER_CRU_STEP,
                         "steps_per_launch": per_launch_steps},
            "issue_roofline": {"warp_inst_per_cru_step": WARP_INST_PER_CRU_STEP,
                               "achieved_warp_inst_per_s": warp_rate,
                               "peak_cell_sms": sms_used * 4 * sm_hz, "frac_cell_sms": warp_rate / (sms_used * 4 * sm_hz),
                               "peak_gpu": 152 * 4 * sm_hz, "frac_gpu": warp_rate / (152 * 4 * sm_hz),
                               "sms_used": sms_used, "sm_hz": sm_hz,
                               "note": "issue slots = 4 schedulers x SM clock per SM; warp instructions per "
                                       "CRU-step from the ncu instruction mix of this workload"},
            "clocks": clocks, "wall_s": wall}
    e.close()
    if rank == 0 and not args.no_extras:
        del flush
        line["e2e"] = e2e_measure(K, span)
        line["paths"] = {"plain_gpu": plain_measure(local_rank, windows),
                         "batched_gpu": batched_measure(local_rank),
                         "config5_gpu": config5_measure(local_rank),
                         "config1_fp64": config1_measure(local_rank)}
        line["accuracy"] = {"fp32_vs_fp64_oracle_crn": accuracy_crn(local_rank, windows, K, span),
                            "fp32_vs_fp64_ensemble": accuracy_ks(local_rank)}
        line["cpu_baseline"] = cpu_baseline(K, span, args.cpu_seconds)
        cpu = line["cpu_baseline"]["value"]
        line["paths"]["cpu"] = {"cru_steps_per_s": cpu, "sim_ms_per_wall_s": cpu / NCRU * DT,
                                "cores": line["cpu_baseline"]["cores"]}
        b = line["paths"]["batched_gpu"]["cru_steps_per_s"]
        line["ratios"] = {"batched_over_plain_launch_per_step": b / line["paths"]["plain_gpu"]["cru_steps_per_s"],
                          "batched_over_single_cell": b / value, "batched_over_cpu": b / cpu,
                          "single_cell_over_cpu": value / cpu, "e2e_over_cpu": line["e2e"]["value"] / cpu}
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def plain_measure(device, windows, steps=200):
    """The paced cell with one engine launch (and one host synchronisation) per global step, timed
    from each window start of the beat (the headline run's checkpoints) for `steps` steps."""
    from gwgb300 import Ensemble

    e = Ensemble([NCRU], precision="fp32", seed=1000, device=device, steps_per_launch=1)
    e.set_pulse(0.0, PERIOD, STIM_DUR, STIM_AMP)
    e.restore(0, windows[0])
    e.run(DT, 50)
    wall = 0.0
    kern = 0.0
    for ck in windows:
        e.restore(0, ck)
        st0 = e.stats()
        t0 = time.perf_counter()
        e.run(DT, steps)
        wall += time.perf_counter() - t0
        kern += (e.stats()["kernel_ms"] - st0["kernel_ms"]) / 1e3
    e.close()
    n = NCRU * steps * len(windows)
    return {"cru_steps_per_s": n / wall, "sim_ms_per_wall_s": steps * len(windows) * DT / wall,
            "kernel_cru_steps_per_s": n / kern,
            "workload": f"1 cell x {NCRU} CRUs, 1 launch + 1 host sync per global step, {steps} steps from each "
                        f"of {len(windows)} window starts across the beat, wall clock"}


def lognormal_params(rng, n_cells, sigma):
    """Per-cell PCaL, GKr, GKs, Vmaxf = Vmaxr and rRyR scaled by log-normal(sigma) factors."""
    from gwgb300 import _lib

    params = []
    for _ in range(n_cells):
        p = _lib.default_params()
        f = rng.lognormal(0.0, sigma, size=5)
        p.PCaL *= f[0]
        p.GKr *= f[1]
        p.GKs *= f[2]
        p.Vmaxf *= f[3]
        p.Vmaxr *= f[3]
        p.rRyR *= f[4]
        params.append(p)
    return params


def batched_config(seed=3, n_cells=256):
    """256 cells, CRU counts uniform in 2,000..12,500, per-cell log-normal(0.1) parameters, cycle
    lengths uniform in 400..1000 ms."""
    import numpy as np

    rng = np.random.default_rng(seed)
    ncru = rng.integers(2000, 12501, size=n_cells)
    params = lognormal_params(rng, n_cells, 0.1)
    cl = rng.uniform(400.0, 1000.0, size=n_cells)
    return ncru, params, cl


def batched_measure(device, window_ms=400.0, cluster_ctas="auto"):
    """Config 3 over 0-400 ms of every cell's first beat (upstroke, release, plateau,
    repolarisation; a whole beat for the cells paced at 400 ms)."""
    from gwgb300 import Ensemble

    ncru, params, cl = batched_config()
    e = Ensemble(list(ncru), params, precision="fp32", seed=11, device=device, cluster_ctas=cluster_ctas)
    for c in range(len(ncru)):
        e.sample_initial_crus(c)
        e.set_pulse(0.0, float(cl[c]), STIM_DUR, STIM_AMP, cell=c)
    steps = int(round(window_ms / DT))
    st0 = e.stats()
    t0 = time.perf_counter()
    e.run(DT, steps)
    wall = time.perf_counter() - t0
    st1 = e.stats()
    e.close()
    kern = (st1["kernel_ms"] - st0["kernel_ms"]) / 1e3
    total = int(ncru.sum()) * steps
    return {"cru_steps_per_s": total / kern, "sim_ms_per_wall_s": len(ncru) * steps * DT / kern,
            "wall_cru_steps_per_s": total / wall, "cells": len(ncru), "crus": int(ncru.sum()),
            "algorithmic_GBps": total * BYTES_PER_CRU_STEP / kern / 1e9,
            "autotuned": cluster_ctas == "auto", "tuned_us_per_step": e.tuned_us_per_step,
            "issue_roofline": {"warp_inst_per_cru_step": BATCHED_WARP_INST_PER_CRU_STEP,
                               "frac_gpu": BATCHED_WARP_INST_PER_CRU_STEP * total / kern / (152 * 4 * 2.07e9),
                               "note": "warp instructions per CRU-step from the ncu capture of one launch at "
                                       "20 ms; 152 SMs x 4 schedulers x 2.07 GHz"},
            "dram_bytes_per_cru_step": BATCHED_TRAFFIC_PER_LAUNCH_CRU * (st1["launches"] - st0["launches"])
                                       * int(ncru.sum()) / total,
            "launch_shape": {k: st1[k] for k in ("cluster_ctas", "cta_crus", "threads_per_cta", "n_clusters")},
            "workload": f"{len(ncru)} cells, 2,000-12,500 CRUs, log-normal(0.1) PCaL/GKr/GKs/Vmax/rRyR, "
                        f"CL 400-1000 ms, 0-{window_ms:g} ms of the beat ({steps} steps)"}


def config5_measure(device, cells=1024, ncru=12500, lib_cells=64, strata=16):
    """Config 5: 1,024 cells of 12,500 CRUs (12.8M CRUs), per-cell log-normal(0.15) parameters, 2 Hz
    pacing, timed over a window in which the cells together cover every phase of the beat.

    A phase library comes first: lib_cells cells (their own parameter sets) run one whole 500 ms
    beat and are checkpointed at `strata` evenly spaced phases.  Cell c of the ensemble takes
    parameter set c % lib_cells and the library state at phase (c // lib_cells) * 500 / strata ms
    (time and RNG step included, so it continues its own beat).  The timed window is one stratum
    long (500 / strata ms): over it the strata tile the whole beat once, so the rate is the
    beat-averaged rate of the ensemble, without simulating every cell's beat first."""
    import numpy as np

    from gwgb300 import Ensemble

    if cells % lib_cells:
        raise ValueError("cells must be a multiple of lib_cells")
    period = 500.0
    rng = np.random.default_rng(5)
    params = lognormal_params(rng, lib_cells, 0.15)
    lib = Ensemble([ncru] * lib_cells, params, precision="fp32", seed=17, device=device)
    for c in range(lib_cells):
        lib.sample_initial_crus(c)
    lib.set_pulse(0.0, period, STIM_DUR, STIM_AMP)
    span = int(round(period / strata / DT))
    states = []
    t0 = time.perf_counter()
    for k in range(strata):
        states.append([lib.checkpoint(c) for c in range(lib_cells)])
        lib.run(DT, span)
    lib.close()
    t_lib = time.perf_counter() - t0
    reps = cells // lib_cells
    e = Ensemble([ncru] * cells, [params[c % lib_cells] for c in range(cells)], precision="fp32", seed=19,
                 device=device, cluster_ctas="auto", tune_steps=100)
    e.set_pulse(0.0, period, STIM_DUR, STIM_AMP)
    for c in range(cells):
        e.restore(c, states[(c // lib_cells) % strata][c % lib_cells])
    del states
    st0 = e.stats()
    e.run(DT, span)
    st1 = e.stats()
    e.close()
    kern = (st1["kernel_ms"] - st0["kernel_ms"]) / 1e3
    total = cells * ncru * span
    return {"cru_steps_per_s": total / kern, "sim_ms_per_wall_s": cells * span * DT / kern,
            "algorithmic_GBps": total * BYTES_PER_CRU_STEP / kern / 1e9, "cells": cells, "crus": cells * ncru,
            "events_per_cru_step": (st1["events"] - st0["events"]) / total,
            "launch_shape": {k: st1[k] for k in ("cluster_ctas", "cta_crus", "threads_per_cta", "n_clusters")},
            "phase_library_s": t_lib,
            "workload": f"{cells} cells x {ncru} CRUs, {lib_cells} log-normal(0.15) PCaL/GKr/GKs/Vmax/rRyR sets x "
                        f"{reps} phases, CL {period:g} ms; cells start at {strata} phases spaced "
                        f"{period / strata:g} ms apart (states from a one-beat library run) and the timed "
                        f"{span * DT:g} ms window covers the whole beat once across them"}


def config4_measure(device, ms=400.0, cells=32, ncru=5000, sample_every=500, checkpoint_every=200):
    """Config 4: 32 cells x 5,000 CRUs, one stimulus, `ms` ms; loss = MSE of V sampled every 0.5 ms
    against a target trace from the same cells with the 8 parameters scaled by 1 + U(-0.2, 0.2);
    the pathwise adjoint with a checkpoint every 200 global steps.  Times the target's forward pass,
    the forward pass at the base parameters and the backward pass (device time, CUDA events)."""
    import numpy as np

    from gwgb300 import _lib
    from gwgb300.adjoint import THETA, GradEngine, initial_states, scaled_params

    steps = int(round(ms / DT))
    base = _lib.default_params()
    g0 = np.frombuffer(bytes(_lib.default_globals(py=True)), dtype=np.float64).copy()
    states = initial_states([ncru] * cells, seed=7, device=device)
    kw = dict(n_steps=steps, seed=7, checkpoint_every=checkpoint_every, sample_every=sample_every, device=device)
    scales = 1.0 + np.random.default_rng(4).uniform(-0.2, 0.2, (cells, len(THETA)))
    with GradEngine([ncru] * cells, [scaled_params(base, s) for s in scales], **kw) as t:
        for c in range(cells):
            t.set_state(c, g0, states[c])
        Vt = t.forward()
        target_ms = t.stats()["forward_ms"]
    with GradEngine([ncru] * cells, base, **kw) as e:
        for c in range(cells):
            e.set_state(c, g0, states[c])
        w0 = time.perf_counter()
        V = e.forward()
        w1 = time.perf_counter()
        sens = e.backward(2.0 * (V - Vt) / Vt.size)
        w2 = time.perf_counter()
        st = e.stats()
    crus = cells * ncru * steps
    return {"workload": f"{cells} cells x {ncru} CRUs, {ms:g} ms after one stimulus (+100 pA/pF, 0.5 ms), V "
                        f"sampled every {sample_every * DT:g} ms, checkpoint every {checkpoint_every} steps",
            "steps": steps, "forward_s": st["forward_ms"] / 1e3, "backward_s": st["backward_ms"] / 1e3,
            "target_forward_s": target_ms / 1e3, "wall_forward_s": w1 - w0, "wall_backward_s": w2 - w1,
            "forward_cru_steps_per_s": crus / (st["forward_ms"] / 1e3),
            "gradient_cru_steps_per_s": crus / ((st["forward_ms"] + st["backward_ms"]) / 1e3),
            "backward_over_forward": st["backward_ms"] / st["forward_ms"],
            "events_per_cru_step": st["events"] / crus,
            "checkpoint_GB": st["checkpoint_bytes"] / 1e9, "segment_GB": st["segment_bytes"] / 1e9,
            "loss": float(np.mean((V - Vt) ** 2)),
            "sens_mean_abs": dict(zip(THETA, np.abs(sens).mean(axis=0).tolist()))}


def profile_batched(device, launches):
    """Config 3's ensemble in the shape its autotune picks (clusters of 6 CTAs, the size rule's CTA
    capacity; the planner then gives the CTAs up to 2,336 CRUs) with 100 global steps per launch:
    200 launches bring it to 20 ms (Ca release), then `launches` more.  For ncu:
    -k regex:engine_kernel -s 200 -c <n>."""
    from gwgb300 import Ensemble

    ncru, params, cl = batched_config()
    e = Ensemble(list(ncru), params, precision="fp32", seed=11, device=device, cluster_ctas=6, cta_crus=0,
                 steps_per_launch=100)
    for c in range(len(ncru)):
        e.sample_initial_crus(c)
        e.set_pulse(0.0, float(cl[c]), STIM_DUR, STIM_AMP, cell=c)
    e.run(DT, 200 * 100)
    st0 = e.stats()
    e.run(DT, launches * 100)
    st1 = e.stats()
    e.close()
    total = int(ncru.sum()) * launches * 100
    print(json.dumps({"profile_batched": {"launches": launches, "crus": int(ncru.sum()),
                                          "us_per_step": (st1["kernel_ms"] - st0["kernel_ms"]) * 1e3 / (launches * 100),
                                          "cru_steps_per_s": total / ((st1["kernel_ms"] - st0["kernel_ms"]) / 1e3),
                                          "events_per_cru_step": (st1["events"] - st0["events"]) / total}}),
          flush=True)


def ks_full_cells(device, cells=200, ncru=12500, t_ms=50.0, every=500):
    """Ensemble statistics at the headline cell size: 200 replicate 12,500-CRU cells (one stream
    each), FP32 engine vs FP64 engine (reference arithmetic), the first t_ms ms after a +100 pA/pF
    0.5 ms stimulus, recorded every 0.5 ms with the device's record-time CRU sums.  Two-sample KS
    p-values (alpha = 0.01) of peak Cai, its time, V at the end of the window, and the peak LCC and
    RyR open fractions and their times."""
    import numpy as np
    from scipy.stats import ks_2samp

    from gwgb300 import Ensemble

    steps = int(round(t_ms / DT))
    out, secs = {}, {}
    for prec, seed in (("fp32", 41), ("fp64", 42)):
        e = Ensemble([ncru] * cells, precision=prec, seed=seed, device=device)
        for c in range(cells):
            e.sample_initial_crus(c)
        e.set_pulse(0.0, PERIOD, STIM_DUR, STIM_AMP)
        st0 = e.stats()
        tr = e.run(DT, steps, record_every=every, sums=True)
        secs[prec] = (e.stats()["kernel_ms"] - st0["kernel_ms"]) / 1e3
        e.close()
        t = (np.arange(tr.globals.shape[1]) + 1) * every * DT
        Cai = tr.var("Cai")
        lcc = tr.sum("LCC_open") / (4 * ncru)
        ryr = tr.sum("RyR_open") / (20 * ncru)
        out[prec] = {"peak_Cai": Cai.max(axis=1), "t_peak_Cai": t[Cai.argmax(axis=1)], "V_end": tr.var("V")[:, -1],
                     "peak_LCC_open": lcc.max(axis=1), "t_peak_LCC_open": t[lcc.argmax(axis=1)],
                     "peak_RyR_open": ryr.max(axis=1), "t_peak_RyR_open": t[ryr.argmax(axis=1)]}
    res = {"reference": "FP64 engine (reference arithmetic, bit-exact channel sequences vs the oracle)",
           "cells": cells, "ncru": ncru, "window_ms": t_ms, "alpha": 0.01, "kernel_s": secs, "ks_pvalue": {},
           "rel_diff_of_means": {}, "fp64_mean": {}}
    for k in out["fp32"]:
        a, b = out["fp32"][k], out["fp64"][k]
        res["ks_pvalue"][k] = float(ks_2samp(a, b).pvalue)
        res["rel_diff_of_means"][k] = float(abs(a.mean() - b.mean()) / max(abs(b.mean()), 1e-30))
        res["fp64_mean"][k] = float(b.mean())
    res["all_pass"] = bool(min(res["ks_pvalue"].values()) > 0.01)
    return res


def _lib_globals():
    from gwgb300 import _lib

    return _lib.default_globals()


def config5_accuracy(device, cells=64, ncru=500, beats=10, every=500):
    """Config 5 accuracy: APD90 and peak Cai of every beat of a 64-cell subset, FP32 engine vs FP64
    engine (reference arithmetic), same seeds and parameter sets (log-normal(0.15), as config 5),
    2 Hz for `beats` beats.  The cells hold ncru CRUs standing for NCaRU = 12,500 (CRU_factor
    12,500 / ncru) so that the FP64 runs fit; both precisions see the same cells.  Reports per beat
    and pooled over beats: KS p-values of the two distributions, relative differences of their means
    and standard deviations, and the mean absolute per-cell difference."""
    import numpy as np
    from scipy.stats import ks_2samp

    from gwgb300 import Ensemble, analysis

    period = 500.0
    rng = np.random.default_rng(5)
    params = lognormal_params(rng, cells, 0.15)
    steps = int(round(beats * period / DT))
    per_beat = int(round(period / (every * DT)))
    out, secs = {}, {}
    for prec in ("fp32", "fp64"):
        e = Ensemble([ncru] * cells, params, precision=prec, seed=23, device=device)
        for c in range(cells):
            e.sample_initial_crus(c)
        e.set_pulse(0.0, period, STIM_DUR, STIM_AMP)
        st0 = e.stats()
        tr = e.run(DT, steps, record_every=every)
        secs[prec] = (e.stats()["kernel_ms"] - st0["kernel_ms"]) / 1e3
        e.close()
        V, Cai = tr.var("V"), tr.var("Cai")
        v0 = np.frombuffer(bytes(_lib_globals()), dtype=np.float64)[0]
        apd, pk = [], []
        t = np.arange(per_beat + 1) * every * DT  # from the beat's stimulus onset
        for b in range(beats):
            sl = slice(b * per_beat, (b + 1) * per_beat)
            # the beat's trace with V just before its stimulus in front (the rest level of APD90)
            before = np.full((cells, 1), v0) if b == 0 else V[:, b * per_beat - 1:b * per_beat]
            mk = analysis.ap_markers(t, np.concatenate([before, V[:, sl]], axis=1))
            apd.append(mk["APD90"])
            pk.append(Cai[:, sl].max(axis=1))
        out[prec] = {"APD90": np.array(apd), "peak_Cai": np.array(pk)}

    def compare(a, b):
        return {"ks_pvalue": float(ks_2samp(a.ravel(), b.ravel()).pvalue),
                "rel_diff_mean": float(abs(a.mean() - b.mean()) / abs(b.mean())),
                "rel_diff_std": float(abs(a.std() - b.std()) / max(b.std(), 1e-300)),
                "mean_abs_cell_diff_rel": float(np.mean(np.abs(a - b)) / abs(b.mean()))}

    res = {"reference": "FP64 engine (reference arithmetic, bit-exact channel sequences vs the oracle)",
           "cells": cells, "ncru": ncru, "NCaRU": 12500, "beats": beats, "cycle_ms": period,
           "kernel_s": secs, "pooled": {}, "per_beat": {}}
    for k in ("APD90", "peak_Cai"):
        a, b = out["fp32"][k], out["fp64"][k]
        res["pooled"][k] = compare(a, b)
        res["per_beat"][k] = [compare(a[i], b[i]) for i in range(beats)]
        res["pooled"][k]["fp64_mean"] = float(b.mean())
        res["pooled"][k]["fp64_std"] = float(b.std())
    return res


def config1_measure(device):
    """Config 1 in full: one cell of 1,250 CRUs (NCaRU 12,500), FP64 throughout, one +100 pA/pF
    stimulus of 0.5 ms, 500 ms, seed 0 -- on the GPU (FP64 engine) and on the CPU (the oracle port,
    Release flags, all cores), the reference's own CPU-runnable case."""
    from gwgb300 import Ensemble, _lib, engine

    import pyoracle as po

    n, steps = 1250, 500_000
    e = Ensemble([n], precision="fp64", seed=0, device=device)
    e.sample_initial_crus(0)
    e.set_globals(0, engine.globals_to_array(_lib.default_globals(py=True)))
    e.set_pulse(0.0, 0.0, STIM_DUR, STIM_AMP)
    st0 = e.stats()
    t0 = time.perf_counter()
    e.run(DT, steps)
    wall = time.perf_counter() - t0
    st1 = e.stats()
    e.close()
    kern = (st1["kernel_ms"] - st0["kernel_ms"]) / 1e3
    threads = os.cpu_count() or 1
    po.build()
    po.timed_lib().orc_set_threads(threads)
    m = po.Model(po.default_params(), n, seed=0, timed=True)
    m.sample_initial_crus()
    m.set_globals(po.default_globals(py=True))
    istim = po.pulse_train(steps, DT, STIM_AMP, STIM_DUR)
    t1 = time.perf_counter()
    m.run(DT, istim, 0)
    cpu_s = time.perf_counter() - t1
    return {"gpu_fp64_cru_steps_per_s": n * steps / kern, "gpu_fp64_wall_cru_steps_per_s": n * steps / wall,
            "gpu_sim_ms_per_wall_s": steps * DT / wall,
            "cpu_cru_steps_per_s": n * steps / cpu_s, "cpu_sim_ms_per_wall_s": steps * DT / cpu_s,
            "cpu_cores": threads, "gpu_over_cpu": (n * steps / wall) / (n * steps / cpu_s),
            "launch_shape": {k: st1[k] for k in ("cluster_ctas", "cta_crus", "threads_per_cta", "n_clusters")},
            "workload": "1 cell x 1,250 CRUs (NCaRU 12,500), FP64, +100 pA/pF 0.5 ms, 500 ms, seed 0, in full"}


def phase_checkpoint(device, windows, span, t_ms):
    """The headline cell's state at t_ms: the latest window start at or before it, advanced on a
    copy of the cell."""
    from gwgb300 import Ensemble

    k = min(int(t_ms / (span * DT)), len(windows) - 1)
    extra = int(round(t_ms / DT)) - k * span
    if extra <= 0:
        return windows[k]
    e = Ensemble([NCRU], precision="fp32", seed=1000, device=device)
    e.set_pulse(0.0, PERIOD, STIM_DUR, STIM_AMP)
    e.restore(0, windows[k])
    e.run(DT, extra)
    ck = e.checkpoint(0)
    e.close()
    return ck


def accuracy_crn(device, windows, K, span, steps=200, points_ms=(0.0, 15.0, 150.0, 350.0)):
    """The FP32 path's error against the FP64 oracle at the headline config, from the same 12,500-CRU
    state with common random numbers (the oracle in 24-bit-uniform mode draws the engine's FP32
    uniforms), after 1 and `steps` global steps, at rest before the stimulus, in the Ca release
    (15 ms), on the plateau (150 ms) and in repolarisation (350 ms)."""
    import numpy as np

    import pyoracle as po
    from gwgb300 import Ensemble

    po.build()
    po.lib().orc_set_threads(os.cpu_count() or 1)
    out = []
    for t_ms in points_ms:
        if t_ms >= K * span * DT:
            continue
        ck = phase_checkpoint(device, windows, span, t_ms)
        s = ck["crus"]
        rec = {"t_ms": ck["t"]}
        for n in (1, steps):
            e = Ensemble([NCRU], precision="fp32", seed=1000, device=device)
            e.set_pulse(0.0, PERIOD, STIM_DUR, STIM_AMP)
            e.restore(0, ck)
            e.run(DT, n)
            g32, s32 = e.get_globals(0), e.get_crus(0)
            e.close()
            m = po.Model(po.default_params(), NCRU, seed=1000, umode=po.U24)
            m.set_globals(po.OrcGlobals.from_array(ck["globals"]))
            o = po.CRUArrays(NCRU)
            for key in ("CaSS", "CaJSR", "LCC", "LCC_inactivation", "RyR", "ClCh"):
                setattr(o, key, getattr(s, key))
            m.set_crus(o)
            jl, cl, jt, jx = ck["carry"]
            m.set_fluxes(s.JLCC, np.full((NCRU, 4), jx / (4 * NCRU)), np.full(NCRU, jt / NCRU))
            m.set_step(ck["step"])
            t = ck["t"]
            for _ in range(n):
                m.euler_step(DT, pulse(t))
                t += DT
            g64, s64 = m.globals().to_array(), m.crus()
            same = np.ones(NCRU, bool)
            for key in ("LCC", "LCC_inactivation", "RyR", "ClCh"):
                same &= np.all(getattr(s32, key).reshape(NCRU, -1) == getattr(s64, key).reshape(NCRU, -1), axis=1)
            relg = np.abs(g32 - g64) / np.maximum(np.abs(g64), 1e-300)
            rec[f"after_{n}"] = {
                "globals_max_rel": float(relg.max()), "V_rel": float(relg[0]), "Cai_rel": float(relg[3]),
                "crus_with_other_channel_state": int((~same).sum()),
                "CaSS_max_rel_same_channels": float(np.max(np.abs(s32.CaSS[same] - s64.CaSS[same]) /
                                                           s64.CaSS[same])) if same.any() else None,
                "CaJSR_max_rel_same_channels": float(np.max(np.abs(s32.CaJSR[same] - s64.CaJSR[same]) /
                                                            s64.CaJSR[same])) if same.any() else None}
        out.append(rec)
    return {"reference": "FP64 oracle (C restatement pinned bit-exact to the reference's C++), 24-bit uniforms "
                         "= the engine's draws", "ncru": NCRU, "points": out}


def accuracy_ks(device, cells=64, ncru=500, t_ms=450.0, every=500):
    """FP32 vs FP64 engine (FP64 = reference arithmetic, bit-exact with the oracle): replicate
    ensembles of one paced beat, KS p-values and relative differences of the means of APD90, peak
    Cai, its time and V at 100 ms."""
    import numpy as np
    from scipy.stats import ks_2samp

    from gwgb300 import Ensemble, analysis

    out = {}
    for prec, seed in (("fp32", 31), ("fp64", 32)):
        e = Ensemble([ncru] * cells, precision=prec, seed=seed, device=device)
        for c in range(cells):
            e.sample_initial_crus(c)
        e.set_pulse(0.0, PERIOD, STIM_DUR, STIM_AMP)
        tr = e.run(DT, int(t_ms / DT), record_every=every)
        e.close()
        V, Cai = tr.var("V"), tr.var("Cai")
        t = (np.arange(V.shape[1]) + 1) * every * DT
        mk = analysis.ap_markers(t, V, v_rest=-91.382)
        out[prec] = {"APD90": mk["APD90"], "peak_Cai": Cai.max(axis=1), "t_peak_Cai": t[Cai.argmax(axis=1)],
                     "V_100ms": V[:, int(100.0 / (every * DT)) - 1]}
    res = {"reference": "FP64 engine (reference arithmetic, bit-exact channel sequences vs the oracle)",
           "cells": cells, "ncru": ncru, "window_ms": t_ms, "ks_pvalue": {}, "rel_diff_of_means": {}}
    for k in out["fp32"]:
        a, b = out["fp32"][k], out["fp64"][k]
        res["ks_pvalue"][k] = float(ks_2samp(a, b).pvalue)
        res["rel_diff_of_means"][k] = float(abs(a.mean() - b.mean()) / max(abs(b.mean()), 1e-30))
    return res


def e2e_measure(K, span):
    """The same beat through the reference-facing C ABI: K chained gw_simulate calls of `span` steps
    (host arrays in; per-step stimulus samples at the global t; the last step's state read back and
    passed to the next call; a fresh context per call, as chained run() calls of the reference)."""
    import ctypes as C

    import numpy as np

    import GreensteinWinslow as GW
    from gwgb300 import _lib

    L = _lib.load()
    p = _lib.default_params()
    g = _lib.default_globals(py=True)
    rng = np.random.default_rng(0)
    LCC, LCCi, RyR, ClCh = GW._initial_cru_arrays(NCRU, rng)
    CaSS = np.full((NCRU, 4), 1.45370e-4)
    CaJSR = np.full(NCRU, 0.908408)
    rec_t = np.zeros(2)
    recG = np.zeros((2, 36))
    rCaSS = np.zeros((2, NCRU, 4))
    rCaJSR = np.zeros((2, NCRU))
    rI = [np.zeros((2, NCRU, 4), np.int32) for _ in range(3)]
    rRyR = np.zeros((2, NCRU, 4, 6), np.int32)
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
    ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int32))  # noqa: E731
    # the stimulus at t_i = sum_{k<i} dt (t += dt), window k's samples istim_all[k*span:(k+1)*span]
    istim_all = np.empty(K * span)
    t = 0.0
    for i in range(K * span):
        istim_all[i] = pulse(t)
        t += DT

    def once(k, state):
        CaSS_, CaJSR_, LCC_, LCCi_, RyR_, ClCh_, g_ = state
        tr = _lib.GwTrace()
        tr.max_records = 2
        tr.t, tr.globals, tr.cru_cell = dp(rec_t), dp(recG), 0
        tr.CaSS, tr.CaJSR = dp(rCaSS), dp(rCaJSR)
        tr.LCC, tr.LCC_inactivation, tr.ClCh, tr.RyR = ip(rI[0]), ip(rI[1]), ip(rI[2]), ip(rRyR)
        istim = np.ascontiguousarray(istim_all[k * span:(k + 1) * span])
        rc = L.gw_simulate(C.byref(p), NCRU, DT, span, dp(istim), max(span - 1, 1), dp(CaSS_), dp(CaJSR_), ip(LCC_),
                           ip(LCCi_), ip(RyR_), ip(ClCh_), C.byref(g_), b"xoshiro256++", 1 + k, 1, C.byref(tr))
        _lib.check(rc)
        last = 1 if span > 1 else 0
        gn = _lib.GwGlobals.from_buffer_copy(recG[last].tobytes())
        return (rCaSS[last].copy(), rCaJSR[last].copy(), rI[0][last].copy(), rI[1][last].copy(), rRyR[last].copy(),
                rI[2][last].copy(), gn)

    state0 = (CaSS, CaJSR, LCC, LCCi, RyR, ClCh, g)
    once(0, state0)   # warm-up call (module and context set-up)
    state = state0
    t0 = time.perf_counter()
    for k in range(K):
        state = once(k, state)
    el = time.perf_counter() - t0
    h2d = CaSS.nbytes + CaJSR.nbytes + LCC.nbytes + LCCi.nbytes + RyR.nbytes + ClCh.nbytes + 8 * span + 288
    d2h = rec_t.nbytes + recG.nbytes + rCaSS.nbytes + rCaJSR.nbytes + sum(a.nbytes for a in rI) + rRyR.nbytes
    return {"value": NCRU * span * K / el, "unit": "CRU-steps/s", "h2d_bytes_per_step": int(h2d),
            "d2h_bytes_per_step": int(d2h), "wall_s": el,
            "path": f"gw_simulate (C ABI, host arrays, a fresh context per call), {K} chained calls of {span} steps "
                    f"covering 0-{K * span * DT:g} ms of the beat"}


if __name__ == "__main__":
    sys.exit(main())
