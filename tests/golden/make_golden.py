"""Generate the golden fixtures in tests/golden/ from the reference's own C++.

Runs the reference (lukeoloughlin/GW-model src/includes, compiled unmodified by oracle/Makefile's
`ref` target against the project's Eigen-API shim, with the counter-based draws injected) and
records, for a handful of seeded cases, the initial state, the globals every `rec` steps, and the
final CRU state and flux carry.  Also records known-answer tables: Philox4x32-10 uniforms, the
Constants struct, and per-subunit transition rates for every LCC state across both RyR lumping
thresholds.

Usage (only where the reference sources exist):  python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))
import pyoracle as po  # noqa: E402

# name: (nCRU, steps, rec, seed, init_seed, umode, stimulus (amp, dur, period), param overrides)
CASES = {
    "rest": (32, 2000, 100, 11, 111, po.U53, (0.0, 0.0, 0.0), {}),
    "ap": (48, 4000, 100, 12, 112, po.U53, (100.0, 0.5, 0.0), {}),
    "ap_u24": (48, 4000, 100, 13, 113, po.U24, (100.0, 0.5, 0.0), {}),
    "params": (24, 3000, 100, 14, 114, po.U53, (100.0, 0.5, 0.0),
               {"PCaL": 9.13e-13 * 1.2, "rRyR": 3.92 * 1.1, "GKr": 0.024 * 0.9, "Vmaxf": 0.0002096 * 1.1,
                "Vmaxr": 0.0002096 * 1.1, "GKs": 0.00271 * 0.95}),
    "release": (16, 30000, 500, 15, 115, po.U53, (100.0, 0.5, 0.0), {}),
    "stim35": (20, 6000, 200, 16, 116, po.U53, (35.0, 2.0, 0.0), {"NCaRU": 5000}),
}


def run_case(name):
    n, steps, rec, seed, iseed, umode, (amp, dur, per), over = CASES[name]
    p = po.default_params(**over)
    init = po.initial_crus(p, n, seed=iseed)
    g0 = po.default_globals(py=True)
    istim = po.pulse_train(steps, 1e-3, amp, dur, per)
    r = po.RefModel(p, n, seed=seed, umode=umode)
    r.set_state(g0, init)
    G = []
    for i in range(steps):
        r.euler_step(1e-3, istim[i])
        if (i + 1) % rec == 0:
            G.append(r.state()[0].to_array())
    g, s, (JLCC, Jxfer, Jtr) = r.state()
    consts, cur = r.consts()
    out = dict(ncru=n, steps=steps, rec=rec, seed=seed, umode=umode, amp=amp, dur=dur, period=per,
               param_names=np.array([k for k in over]), param_values=np.array([over[k] for k in over], dtype=float),
               g0=g0.to_array(), globals_rec=np.array(G), globals_final=g.to_array(),
               JLCC=JLCC, Jxfer=Jxfer, Jtr=Jtr,
               consts=np.frombuffer(bytes(consts), dtype=np.float64),
               currents=np.frombuffer(bytes(cur), dtype=np.float64))
    for k, v in init.as_dict().items():
        out["init_" + k] = v
    for k, v in s.as_dict().items():
        out["final_" + k] = v
    return out


def kat_tables():
    L = po.ref_lib()
    p = po.default_params()
    lcc_states, lcci, clch, cass, ryr_cfgs = range(1, 13), (0, 1), (0, 1), \
        (1e-5, 1.0e-4, 1.15e-4, 1.2e-4, 2e-3, 0.03685, 0.04, 0.3), \
        ([5, 0, 0, 0, 0, 0], [1, 1, 1, 1, 1, 0], [0, 2, 1, -1, 3, 0], [3, 0, 0, 0, 1, 1], [0, 0, 4, 1, 0, 0])
    rows = []
    V = -45.3
    for s in lcc_states:
        for li in lcci:
            for ch in clch:
                for x in cass:
                    for rc in ryr_cfgs:
                        LCC = np.array([s, 1 + (s % 12), 7, 12], np.int32)
                        LCCi = np.array([li, 1 - li, 1, 0], np.int32)
                        RyR = np.array(rc * 4, np.int32)
                        ClCh = np.array([ch, 1 - ch, 0, 1], np.int32)
                        CaSS = np.array([x, x * 0.5, x * 2.0, 1.45e-4])
                        o = [np.zeros(12), np.zeros(4), np.zeros(48), np.zeros(4), np.zeros(4)]
                        L.ref_cru_rates(C.byref(p), V, *[a.ctypes.data_as(C.POINTER(C.c_int)) for a in (LCC, LCCi, RyR, ClCh)],
                                        CaSS.ctypes.data_as(C.POINTER(C.c_double)),
                                        *[a.ctypes.data_as(C.POINTER(C.c_double)) for a in o])
                        rows.append((LCC, LCCi, RyR, ClCh, CaSS, *o))
    cols = list(zip(*rows))
    names = ["LCC", "LCCi", "RyR", "ClCh", "CaSS", "LCC_rates", "LCCi_rates", "RyR_rates", "ClCh_rates", "subunit_rates"]
    out = {n: np.array(c) for n, c in zip(names, cols)}
    out["V"] = np.array(V)
    # Constants after one step from the Python default state, for two nCRU values
    for ncru in (1250, 12500):
        r = po.RefModel(p, ncru, seed=1)
        c, _ = r.consts()
        out[f"consts_n{ncru}"] = np.frombuffer(bytes(c), dtype=np.float64).copy()
    # Philox4x32-10 uniforms of a few streams (both modes)
    keys = [(0, 0, 0, 0), (7, 3, 1234, 99), (2**63 + 5, 1023, 2**31 + 7, 4_999_999)]
    out["uni_keys"] = np.array(keys, dtype=np.uint64)
    out["uni_u53"] = np.array([po.uniforms(s, c, k, st, 16, po.U53) for s, c, k, st in keys])
    out["uni_u24"] = np.array([po.uniforms(s, c, k, st, 16, po.U24) for s, c, k, st in keys])
    return out


def main():
    po.build()
    if not po.ref_available():
        raise SystemExit("the reference harness (oracle/_ref) is not built here")
    for name in CASES:
        np.savez_compressed(os.path.join(HERE, f"traj_{name}.npz"), **run_case(name))
        print("wrote", name)
    np.savez_compressed(os.path.join(HERE, "kat_tables.npz"), **kat_tables())
    print("wrote kat_tables")


if __name__ == "__main__":
    main()
