"""The reference-facing run path on the GPU against the oracle, run the reference's way.

The reference's `GreensteinWinslow.run` (src/pyGW.cpp:341-344 -> run_PRNG_arg :134-157 ->
run<PRNG>, src/pyGW.hpp:102-122) builds the model, evaluates the Python stimulus callable at the
accumulated t (t += step_size, pyGW.hpp:110-116), steps, and after every step i with
i % record_every == 0 records t, the 36 globals and every CRU array (record_state,
pyGW.hpp:56-99).  The oracle's `run_record` is that loop; here the drop-in module and the C ABI
(`gw_simulate`) run it on the GB300 engine in FP64 and every record is compared:

  t                      bit-exact (both sides accumulate t += dt in FP64)
  channel states         bit-exact (LCC, LCC_inactivation, RyR, ClCh of every CRU, every record)
  CaSS, CaJSR, globals   within 1e-12 relative
  CaSS over 500,000 steps (config 1) within 1e-11 relative: one step from an identical state agrees
                         to 1e-12 (tests/test_gpu_parity.py), but over a whole beat the 1-ulp
                         differences of the device's FP64 log (jump times) and exp (per-step rate
                         constants) add up in CRUs with thousands of events; measured on GB300: every
                         CaSS within 4e-14 except one subunit beside an open RyR mid-release (27 ms)
                         at 1.6e-12, globals within 1.4e-13, CaJSR within 6e-16

The reference allocates num_steps // record_every records (pyGW.hpp:109) and writes one more when
record_every does not divide num_steps; the drop-in keeps the allocated ones, and the oracle
reports how many the reference's loop makes.

Initial JLCC: the reference's constructor computes JLCC from its own random CRU state
(GW.hpp:104-112), whose LCC states are 1, 2 or 7 (GW_utils.tpp:5-64), never the open states 6
and 12, so JLCC starts at zero whatever initial state `set_initial_value` installs afterwards.
The engine starts from JLCC = 0 as well; the initial states below hold open LCCs to exercise it.
"""
import ctypes as C
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CHANNELS = ("LCC", "LCC_inactivation", "RyR", "ClCh")
RTOL = 1e-12


def rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300))) if a.size else 0.0


def sample(fn, n, dt):
    """A stimulus callable evaluated at t_i = sum_{k<i} dt, as the reference's loop does."""
    out = np.empty(n)
    t = 0.0
    for i in range(n):
        out[i] = fn(t)
        t += dt
    return out


def open_lcc_state(po, p, n, seed):
    """The reference's random initial CRU state with a share of subunits moved to the open LCC
    states (6 and 12) with the voltage gate not inactivated, and raised subspace Ca."""
    s = po.initial_crus(p, n, seed=seed)
    rng = np.random.default_rng(seed)
    pick = rng.random((n, 4)) < 0.15
    s.LCC[pick] = rng.choice([6, 12], size=int(pick.sum()))
    s.LCC_inactivation[pick] = 1
    s.CaSS = s.CaSS * (1.0 + rng.random((n, 4)))
    return s


def check_records(po_rec, t, G, crus, R, cass_rtol=RTOL):
    assert t.shape == (R,) and G.shape == (R, 36)
    np.testing.assert_array_equal(t, po_rec["t"])
    assert rel(G, po_rec["globals"]) <= RTOL
    for k in CHANNELS:
        np.testing.assert_array_equal(crus[k], po_rec[k], err_msg=k)
    assert rel(crus["CaSS"], po_rec["CaSS"]) <= cass_rtol
    assert rel(crus["CaJSR"], po_rec["CaJSR"]) <= RTOL


@pytest.mark.parametrize("num_steps,record_every", [(4000, 250), (4000, 7), (2999, 1000), (1500, 1)])
def test_dropin_run_matches_reference_loop(oracle, GW, num_steps, record_every):
    """GreensteinWinslow.run with a Python stimulus callable, FP64, an initial state with open LCCs."""
    po = oracle
    n, dt, seed = 120, 1e-3, 21
    p = po.default_params()
    init = open_lcc_state(po, p, n, seed=5)
    fn = lambda t: 100.0 if t < 0.5 else 0.0  # noqa: E731
    m = po.Model(p, n, seed=seed)
    m.set_globals(po.default_globals(py=True))
    m.set_crus(init)
    made, ref = m.run_record(dt, sample(fn, num_steps, dt), record_every)
    R = num_steps // record_every
    assert made == -(-num_steps // record_every)

    ic = GW.GWCRUState(n)
    for k in ("CaSS", "CaJSR") + CHANNELS:
        setattr(ic, k, getattr(init, k))
    out = GW.run(GW.GWParameters(), n, dt, num_steps, fn, record_every, ic, GW.GWGlobalState(),
                 "xoshiro256++", seed=seed, precision="fp64")
    G = np.concatenate([np.stack([getattr(out, k) for k in ("V", "Nai", "Ki", "Cai", "CaNSR", "CaLTRPN",
                                                              "CaHTRPN", "m", "h", "j", "xKs")], axis=1),
                        out.XKr, out.XKv43, out.XKv14], axis=1)
    check_records(ref, out.t, G, {k: getattr(out, k) for k in ("CaSS", "CaJSR") + CHANNELS}, R)
    assert out.CaSS.shape == (R, n, 4) and out.RyR.shape == (R, n, 4, 6)


def _simulate(L, _lib, p, n, dt, istim, record_every, init, g0, seed, precision=0):
    """gw_simulate through the C ABI with host arrays, recording every CRU array."""
    steps = istim.size
    R = steps // record_every
    out = {"t": np.zeros(R), "G": np.zeros((R, 36)), "CaSS": np.zeros((R, n, 4)), "CaJSR": np.zeros((R, n)),
           "LCC": np.zeros((R, n, 4), np.int32), "LCC_inactivation": np.zeros((R, n, 4), np.int32),
           "RyR": np.zeros((R, n, 4, 6), np.int32), "ClCh": np.zeros((R, n, 4), np.int32)}
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
    ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int32))  # noqa: E731
    tr = _lib.GwTrace()
    tr.max_records = R
    tr.t, tr.globals, tr.cru_cell = dp(out["t"]), dp(out["G"]), 0
    tr.CaSS, tr.CaJSR = dp(out["CaSS"]), dp(out["CaJSR"])
    tr.LCC, tr.LCC_inactivation = ip(out["LCC"]), ip(out["LCC_inactivation"])
    tr.RyR, tr.ClCh = ip(out["RyR"]), ip(out["ClCh"])
    a = {k: np.ascontiguousarray(getattr(init, k), np.int32 if k in CHANNELS else np.float64)
         for k in ("CaSS", "CaJSR") + CHANNELS}
    gp = _lib.GwParams.from_buffer_copy(bytes(p))
    gg = _lib.GwGlobals.from_buffer_copy(bytes(g0))
    rc = L.gw_simulate(C.byref(gp), n, dt, steps, dp(istim), record_every, dp(a["CaSS"]), dp(a["CaJSR"]),
                       ip(a["LCC"]), ip(a["LCC_inactivation"]), ip(a["RyR"]), ip(a["ClCh"]), C.byref(gg),
                       b"mt19937_64", seed, precision, C.byref(tr))
    _lib.check(rc)
    assert tr.n_written == R
    return out


def test_gw_simulate_config1_full(oracle, enginelib):
    """Config 1 in full through the C ABI: 1,250 CRUs standing for NCaRU = 12,500 (CRU_factor 10),
    reference default parameters, GWGlobalState() resting globals, the reference's random initial
    CRU state, dt = 1e-3 ms, one +100 pA/pF stimulus of 0.5 ms (the reference integrates
    dV = dt (Istim - sum I)), 500 ms (500,000 steps), seed 0, FP64 throughout; records every
    3,000 steps (166 kept, the reference's loop makes 167)."""
    from gwgb300 import _lib

    po = oracle
    po.lib().orc_set_threads(os.cpu_count() or 1)
    n, dt, steps, every, seed = 1250, 1e-3, 500_000, 3000, 0
    p = po.default_params()
    assert p.NCaRU == 12500
    init = po.initial_crus(p, n, seed=seed)
    g0 = po.default_globals(py=True)
    istim = po.pulse_train(steps, dt, 100.0, 0.5)
    m = po.Model(p, n, seed=seed)
    m.set_globals(g0)
    m.set_crus(init)
    made, ref = m.run_record(dt, istim, every)
    assert made == 167 and ref["t"].size == 166
    out = _simulate(enginelib, _lib, p, n, dt, istim, every, init, g0, seed)
    check_records(ref, out["t"], out["G"], out, 166, cass_rtol=1e-11)
    # the beat happened: upstroke above 0 mV and Ca release in the records
    V = ref["globals"][:, 0]
    assert V.max() > 0.0 and ref["globals"][:, 3].max() > 3 * g0.Cai


def test_gw_simulate_open_lcc_init(oracle, enginelib):
    """gw_simulate from an initial state with open LCCs (initial JLCC zero, as the reference's ctor
    leaves it) and a non-default parameter set, recorded every step for the first 40 steps."""
    from gwgb300 import _lib

    po = oracle
    n, dt, seed = 64, 1e-3, 7
    p = po.default_params(PCaL=9.13e-13 * 1.3, rRyR=3.92 * 0.9, NCaRU=6400)
    init = open_lcc_state(po, p, n, seed=8)
    g0 = po.default_globals(py=True)
    istim = po.pulse_train(40, dt, 100.0, 0.5)
    m = po.Model(p, n, seed=seed)
    m.set_globals(g0)
    m.set_crus(init)
    made, ref = m.run_record(dt, istim, 1)
    out = _simulate(enginelib, _lib, p, n, dt, istim, 1, init, g0, seed)
    check_records(ref, out["t"], out["G"], out, 40)
