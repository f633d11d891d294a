"""Benchmark: CRU-steps/s and simulated ms per wall-second of the Greenstein-Winslow hybrid SSA,
batched GPU vs plain GPU vs the reference's CPU path.

Workload of the JSON line's `value` (one GPU): one full cell of 12,500 CRUs (NCaRU = 12,500, so
each simulated CRU stands for one real CRU), reference default parameters, GW::GlobalState resting
globals, the reference's random initial CRU distributions, dt = 1e-3 ms, 1 Hz pacing with a
+100 pA/pF, 0.5 ms stimulus (the reference integrates dV = dt (Istim - sum I), so the usual
-100 pA/pF inward stimulus is +100 here).  CRU state FP32, global ODE FP64 with compensated flux
reduction.  Synthetic seeded input.  A bench step is `--span-ms` of simulated time of that paced
cell; the timed steps continue the protocol.

  value        CRU-steps/s, state resident on the device, CUDA events around the engine kernel
  e2e          the same through the reference-facing C ABI (gw_simulate: host arrays in and out,
               the per-step stimulus samples uploaded, a fresh context per call)
  paths        plain GPU (the same cell, one kernel launch per global step) and batched GPU (256
               cells of 2,000-12,500 CRUs, log-normal per-cell parameters and 400-1000 ms cycle
               lengths in one launch), each as CRU-steps/s and simulated ms per wall-second
  roofline     the engine kernel against HBM, algorithmic bytes = the 72-byte FP32 CRU state read
               and written once per CRU-step; the kernel keeps the state on chip between steps, so
               the bound that binds is the per-step dependency chain (see profiles/)
  cpu_baseline the oracle port of the reference's C++ (OpenMP over CRUs) on the host cores,
               bounded sample

--impl reference times the reference's CPU implementation of the path (the oracle port) on the
host cores with all threads.
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
# DRAM bytes (read + write) of one 1000-step launch of this workload, from the ncu capture in
# profiles/engine_kernel_cell12500.txt (the bench's launches have exactly that shape).
TRAFFIC_PER_LAUNCH = 1.047296e6


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--span-ms", type=float, default=20.0)
    ap.add_argument("--cells", type=int, default=1, help="replicate cells per GPU (1 = plain path)")
    ap.add_argument("--no-extras", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
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


def peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def cpu_baseline(seconds: float, ncru: int = NCRU):
    """The oracle port (C restatement of the reference, OpenMP over CRUs) timed on the host cores on
    a bounded sample of the paced cell: the first steps after the stimulus."""
    import pyoracle as po

    po.build()
    threads = os.cpu_count() or 1
    po.lib().orc_set_threads(threads)
    p = po.default_params()
    m = po.Model(p, ncru, seed=0)
    m.sample_initial_crus()
    m.set_globals(po.default_globals(py=False))
    t0 = time.perf_counter()
    steps = 0
    t = 0.0
    while True:
        tb = t - PERIOD * float(int(t / PERIOD))
        m.euler_step(DT, STIM_AMP if tb < STIM_DUR else 0.0)
        t += DT
        steps += 1
        el = time.perf_counter() - t0
        if el >= seconds:
            break
    rate = ncru * steps / el
    return {"value": rate, "unit": "CRU-steps/s", "cores": threads, "kind": "port",
            "sample": f"{ncru} CRUs x {steps} steps ({steps * DT:.3f} ms from the stimulus) in {el:.1f} s"}


def workload_config(args, world=1):
    cells = max(args.cells, 1)
    return {"workload": f"{'single cell' if cells == 1 else f'{cells} replicate cells'} of {NCRU} CRUs, "
                        f"1 Hz pacing (+{STIM_AMP:g} pA/pF, {STIM_DUR:g} ms), dt 1e-3 ms, "
                        f"FP32 CRU state, FP64 global ODE",
            "ncru": NCRU, "cells_per_gpu": cells, "span_ms_per_step": args.span_ms,
            "parallelism": f"replicas x{world}",
            "l2": "CRU state (0.9 MB per cell) stays in shared memory across steps; no L2 flush"}


def run_reference(args):
    from gwgb300 import dist as gd

    rank, _, world = gd.env_rank()
    if rank != 0:
        return 0
    K, W = args.steps, args.warmup
    per = max(args.cpu_seconds / max(K + W, 1), 2.0)
    for _ in range(W):
        cpu_baseline(per)
    vals = [cpu_baseline(per) for _ in range(K)]
    v = statistics.median(x["value"] for x in vals)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "CRU-steps/s",
            "n_gpus": args.gpus, "steps": K, "warmup": W, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(args, world),
            "cpu_baseline": {"value": v, "unit": "CRU-steps/s", "cores": vals[0]["cores"], "kind": "port",
                             "sample": vals[0]["sample"]},
            "e2e": {"value": v, "unit": "CRU-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    import numpy as np

    from gwgb300 import Ensemble
    from gwgb300 import dist as gd

    rank, local_rank, world = gd.env_rank()
    d = gd.init()
    span = int(round(args.span_ms / DT))
    K, W = args.steps, max(args.warmup, 3)
    cells = max(args.cells, 1)
    e = Ensemble([NCRU] * cells, precision="fp32", seed=1000 + rank, device=local_rank)
    for c in range(cells):
        e.sample_initial_crus(c)
    e.set_pulse(0.0, PERIOD, STIM_DUR, STIM_AMP)
    for _ in range(W):
        e.run(DT, span)
    gd.barrier(d)
    st0 = e.stats()
    t0 = time.perf_counter()
    with ClockSampler(local_rank) as clk:
        for _ in range(K):
            e.run(DT, span)
    wall = time.perf_counter() - t0
    st1 = e.stats()
    kernel_s = (st1["kernel_ms"] - st0["kernel_ms"]) / 1e3
    kernel_s = gd.max_over_ranks(d, kernel_s)
    wall = gd.max_over_ranks(d, wall)
    cru_steps = NCRU * cells * span * K * world
    value = cru_steps / kernel_s
    launches = int(st1["launches"] - st0["launches"])
    pk, pk_kind = peaks()
    per_launch_steps = span * K / max(launches, 1)
    achieved_gbs = BYTES_PER_CRU_STEP * NCRU * cells * span * K / kernel_s / 1e9
    line = {"metric": METRIC, "value": value, "unit": "CRU-steps/s", "n_gpus": world,
            "steps": K, "warmup": W, "ms_per_step": kernel_s / K * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(args, world),
            "launch_shape": {k: st1[k] for k in ("cluster_ctas", "cta_crus", "threads_per_cta", "n_clusters")},
            "sim_ms_per_wall_s": cells * world * span * K * DT / kernel_s,
            "events_per_cru_step": (st1["events"] - st0["events"]) / max(NCRU * cells * span * K, 1),
            "gpu_launches": launches,
            "roofline": {"bound": "hbm", "achieved": achieved_gbs, "peak": pk["hbm_gbs"], "unit": "GB/s",
                         "frac": achieved_gbs / pk["hbm_gbs"],
                         "traffic": TRAFFIC_PER_LAUNCH if per_launch_steps == 1000 and cells == 1 else None,
                         "traffic_unit": "bytes per launch (ncu dram read + write)",
                         "peak_kind": pk_kind, "bytes_per_cru_step": BYTES_PER_CRU_STEP,
                         "steps_per_launch": per_launch_steps},
            "clocks": clk.summary(), "wall_s": wall}
    e.close()
    if rank == 0 and not args.no_extras:
        line["e2e"] = e2e_measure(span, K)
        line["paths"] = {"plain_gpu": plain_measure(local_rank), "batched_gpu": batched_measure(local_rank),
                         "large_ensemble_gpu": large_measure(local_rank)}
        line["accuracy"] = accuracy_vs_fp64(local_rank)
        line["cpu_baseline"] = cpu_baseline(args.cpu_seconds)
        line["paths"]["cpu"] = {"cru_steps_per_s": line["cpu_baseline"]["value"],
                                "sim_ms_per_wall_s": line["cpu_baseline"]["value"] / NCRU * DT,
                                "cores": line["cpu_baseline"]["cores"]}
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def plain_measure(device, steps=3000):
    """The same paced cell with one engine launch (and one host synchronisation) per global step."""
    from gwgb300 import Ensemble

    e = Ensemble([NCRU], precision="fp32", seed=7, device=device, steps_per_launch=1)
    e.sample_initial_crus(0)
    e.set_pulse(0.0, PERIOD, STIM_DUR, STIM_AMP)
    e.run(DT, 300)
    st0 = e.stats()
    t0 = time.perf_counter()
    e.run(DT, steps)
    wall = time.perf_counter() - t0
    st1 = e.stats()
    e.close()
    kern = (st1["kernel_ms"] - st0["kernel_ms"]) / 1e3
    return {"cru_steps_per_s": NCRU * steps / wall, "sim_ms_per_wall_s": steps * DT / wall,
            "kernel_cru_steps_per_s": NCRU * steps / kern, "launches": int(st1["launches"] - st0["launches"]),
            "workload": f"1 cell x {NCRU} CRUs, 1 launch per global step, {steps} steps, wall clock"}


def batched_config(seed=3, n_cells=256):
    """256 cells, CRU counts uniform in 2,000..12,500, per-cell PCaL, GKr, GKs, Vmaxf = Vmaxr and
    rRyR scaled by log-normal(sigma 0.1) factors, cycle lengths uniform in 400..1000 ms."""
    import numpy as np

    from gwgb300 import _lib

    rng = np.random.default_rng(seed)
    ncru = rng.integers(2000, 12501, size=n_cells)
    params = []
    for _ in range(n_cells):
        p = _lib.default_params()
        f = rng.lognormal(0.0, 0.1, size=5)
        p.PCaL *= f[0]
        p.GKr *= f[1]
        p.GKs *= f[2]
        p.Vmaxf *= f[3]
        p.Vmaxr *= f[3]
        p.rRyR *= f[4]
        params.append(p)
    cl = rng.uniform(400.0, 1000.0, size=n_cells)
    return ncru, params, cl


def batched_measure(device, steps=2000, cluster_ctas="auto"):
    from gwgb300 import Ensemble

    ncru, params, cl = batched_config()
    e = Ensemble(list(ncru), params, precision="fp32", seed=11, device=device, cluster_ctas=cluster_ctas)
    for c in range(len(ncru)):
        e.sample_initial_crus(c)
        e.set_pulse(0.0, float(cl[c]), STIM_DUR, STIM_AMP, cell=c)
    e.run(DT, 500)
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
            "autotuned": cluster_ctas == "auto",
            "launch_shape": {k: st1[k] for k in ("cluster_ctas", "cta_crus", "threads_per_cta", "n_clusters")},
            "workload": f"{len(ncru)} cells, 2,000-12,500 CRUs, log-normal(0.1) PCaL/GKr/GKs/Vmax/rRyR, "
                        f"CL 400-1000 ms, {steps} steps"}


def accuracy_vs_fp64(device, cells=64, ncru=200, t_ms=200.0):
    """Error of the FP32 engine (the measured path) against the FP64 engine (reference arithmetic,
    checked bit-exact against the oracle): replicate-cell ensembles of one paced beat, two-sample
    KS p-values and relative differences of the ensemble means of peak Cai, its time and V."""
    import numpy as np
    from scipy.stats import ks_2samp

    from gwgb300 import Ensemble

    every = 500
    out = {}
    for prec, seed in (("fp32", 31), ("fp64", 32)):
        e = Ensemble([ncru] * cells, precision=prec, seed=seed, device=device)
        for c in range(cells):
            e.sample_initial_crus(c)
        e.set_pulse(0.0, PERIOD, STIM_DUR, STIM_AMP)
        tr = e.run(DT, int(t_ms / DT), record_every=every)
        e.close()
        V, Cai = tr.var("V"), tr.var("Cai")
        i100 = int(100.0 / (every * DT)) - 1
        out[prec] = {"peak_Cai": Cai.max(axis=1), "t_peak_Cai": Cai.argmax(axis=1) * every * DT,
                     "V_100ms": V[:, i100], "Cai_150ms": Cai[:, int(150.0 / (every * DT)) - 1]}
    res = {"reference": "FP64 engine (reference arithmetic)", "cells": cells, "ncru": ncru,
           "window_ms": t_ms, "ks_pvalue": {}, "rel_diff_of_means": {}}
    for k in out["fp32"]:
        a, b = out["fp32"][k], out["fp64"][k]
        res["ks_pvalue"][k] = float(ks_2samp(a, b).pvalue)
        res["rel_diff_of_means"][k] = float(abs(a.mean() - b.mean()) / max(abs(b.mean()), 1e-30))
    return res


def large_measure(device, cells=1024, ncru=12500, steps=1000):
    """Large ensemble: 1,024 cells of 12,500 CRUs (12.8M CRUs), per-cell PCaL, GKr, GKs,
    Vmaxf = Vmaxr and rRyR scaled by log-normal(sigma 0.15) factors, 2 Hz pacing (CL 500 ms)."""
    import numpy as np

    from gwgb300 import Ensemble, _lib

    rng = np.random.default_rng(5)
    params = []
    for _ in range(cells):
        p = _lib.default_params()
        f = rng.lognormal(0.0, 0.15, size=5)
        p.PCaL *= f[0]
        p.GKr *= f[1]
        p.GKs *= f[2]
        p.Vmaxf *= f[3]
        p.Vmaxr *= f[3]
        p.rRyR *= f[4]
        params.append(p)
    e = Ensemble([ncru] * cells, params, precision="fp32", seed=17, device=device, cluster_ctas="auto",
                 tune_steps=100)
    for c in range(cells):
        e.sample_initial_crus(c)
    e.set_pulse(0.0, 500.0, STIM_DUR, STIM_AMP)
    e.run(DT, 200)
    st0 = e.stats()
    e.run(DT, steps)
    st1 = e.stats()
    e.close()
    kern = (st1["kernel_ms"] - st0["kernel_ms"]) / 1e3
    total = cells * ncru * steps
    return {"cru_steps_per_s": total / kern, "sim_ms_per_wall_s": cells * steps * DT / kern,
            "algorithmic_GBps": total * BYTES_PER_CRU_STEP / kern / 1e9, "cells": cells, "crus": cells * ncru,
            "launch_shape": {k: st1[k] for k in ("cluster_ctas", "cta_crus", "threads_per_cta", "n_clusters")},
            "workload": f"{cells} cells x {ncru} CRUs, log-normal(0.15) PCaL/GKr/GKs/Vmax/rRyR, CL 500 ms, {steps} steps"}


def e2e_measure(span, K):
    """The reference-facing path: GreensteinWinslow.run-equivalent C call with host buffers."""
    import ctypes as C

    import numpy as np

    from gwgb300 import _lib

    L = _lib.load()
    p = _lib.default_params()
    g = _lib.default_globals(py=True)
    import GreensteinWinslow as GW

    rng = np.random.default_rng(0)
    LCC, LCCi, RyR, ClCh = GW._initial_cru_arrays(NCRU, rng)
    CaSS = np.full((NCRU, 4), 1.45370e-4)
    CaJSR = np.full(NCRU, 0.908408)
    t = np.arange(span) * DT
    istim = np.where(t - PERIOD * np.floor(t / PERIOD) < STIM_DUR, STIM_AMP, 0.0)
    rec_every = span
    out = {k: np.zeros((1, NCRU, 4)) for k in ("CaSS",)}
    tr = _lib.GwTrace()
    rec_t = np.zeros(1)
    recG = np.zeros(36)
    rCaSS = np.zeros((1, NCRU, 4))
    rCaJSR = np.zeros((1, NCRU))
    rI = [np.zeros((1, NCRU, 4), np.int32) for _ in range(3)]
    rRyR = np.zeros((1, NCRU, 4, 6), np.int32)
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int32))

    def once():
        tr.max_records = 1
        tr.t, tr.globals, tr.cru_cell = dp(rec_t), dp(recG), 0
        tr.CaSS, tr.CaJSR = dp(rCaSS), dp(rCaJSR)
        tr.LCC, tr.LCC_inactivation, tr.ClCh, tr.RyR = ip(rI[0]), ip(rI[1]), ip(rI[2]), ip(rRyR)
        rc = L.gw_simulate(C.byref(p), NCRU, DT, span, dp(istim), rec_every, dp(CaSS), dp(CaJSR), ip(LCC),
                           ip(LCCi), ip(RyR), ip(ClCh), C.byref(g), b"xoshiro256++", 1, 1, C.byref(tr))
        _lib.check(rc)

    once()
    t0 = time.perf_counter()
    for _ in range(K):
        once()
    el = time.perf_counter() - t0
    h2d = CaSS.nbytes + CaJSR.nbytes + LCC.nbytes + LCCi.nbytes + RyR.nbytes + ClCh.nbytes + istim.nbytes
    d2h = rec_t.nbytes + recG.nbytes + rCaSS.nbytes + rCaJSR.nbytes + sum(a.nbytes for a in rI) + rRyR.nbytes
    return {"value": NCRU * span * K / el, "unit": "CRU-steps/s", "h2d_bytes_per_step": int(h2d),
            "d2h_bytes_per_step": int(d2h), "path": "gw_simulate (C ABI, host arrays, fresh context per call)"}


if __name__ == "__main__":
    sys.exit(main())
