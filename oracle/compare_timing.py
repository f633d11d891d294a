"""CPU speed of the oracle port against the reference's own C++ on the same cores (TEST AND CPU-BASELINE
INFRASTRUCTURE ONLY; needs oracle/_ref, which exists only where the reference sources were built).

Workload, the same for all three builds: one cell of --ncru CRUs with the reference's random
initial CRU state and GW::GlobalState defaults, dt = 1e-3 ms, 1 Hz pacing (+100 pA/pF for 0.5 ms),
--steps global steps from t = 0, OpenMP over CRUs on --threads threads (default: all cores).

  port (parity build)   oracle/_build/liboracle.so        -O2 -fno-fast-math -ffp-contract=off
  port (Release build)  oracle/_build/liboracle_timed.so  -Ofast -funroll-loops
  reference (Release)   oracle/_ref/libgwref_timed.so     the reference's GW_model<double,
                        Xoshiro256PlusPlus>::euler_step, unmodified, -Ofast -march=native
                        -funroll-loops (src/CMakeLists.txt:25-34)

Usage:  python oracle/compare_timing.py [--ncru 12500] [--steps 3000] [--threads N] [--repeat 3]
Prints one JSON line with CRU-steps/s of each build and the ratios.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import time

import pyoracle as po


def time_port(timed: bool, ncru: int, steps: int, threads: int) -> float:
    L = po.timed_lib() if timed else po.lib()
    L.orc_set_threads(threads)
    p = po.default_params()
    m = po.Model(p, ncru, seed=1, timed=timed)
    m.sample_initial_crus()
    m.set_globals(po.default_globals(py=False))
    istim = po.pulse_train(steps, 1e-3, 100.0, 0.5, 1000.0)
    t0 = time.perf_counter()
    for i in range(steps):
        m.euler_step(1e-3, istim[i])
    return time.perf_counter() - t0


def time_reference(ncru: int, steps: int, threads: int) -> float:
    L = C.CDLL(po.REF_TIMED_PATH)
    L.ref_time_xoshiro.restype = C.c_double
    L.ref_time_xoshiro.argtypes = [C.POINTER(po.OrcParams), C.c_int, C.c_double, C.c_longlong, C.c_double,
                                   C.c_double, C.c_double, C.c_int]
    p = po.default_params()
    return L.ref_time_xoshiro(C.byref(p), ncru, 1e-3, steps, 1000.0, 0.5, 100.0, threads)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ncru", type=int, default=12500)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--repeat", type=int, default=3)
    a = ap.parse_args()
    po.build()
    work = a.ncru * a.steps
    best = {}
    for name, fn in (("port_parity", lambda: time_port(False, a.ncru, a.steps, a.threads)),
                     ("port_release", lambda: time_port(True, a.ncru, a.steps, a.threads)),
                     ("reference_release", lambda: time_reference(a.ncru, a.steps, a.threads))):
        if name == "reference_release" and not os.path.exists(po.REF_TIMED_PATH):
            continue
        best[name] = work / min(fn() for _ in range(a.repeat))
    out = {"ncru": a.ncru, "steps": a.steps, "threads": a.threads, "cru_steps_per_s": best}
    if "reference_release" in best:
        out["port_release_over_reference"] = best["port_release"] / best["reference_release"]
        out["port_parity_over_reference"] = best["port_parity"] / best["reference_release"]
    print(json.dumps(out))


if __name__ == "__main__":
    main()
