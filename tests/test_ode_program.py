"""The engine's SIMT lane program for the global step (evaluated on the host in the device's
operation order) against the oracle's euler_step (GW.tpp:237-272): one step from many states,
both gate-rate regimes (V >= -40 and V < -40), default and general Jup exponents."""
import ctypes as C

import numpy as np
import pytest


def _states(oracle, seed, n=24):
    """Globals along an oracle AP (rest, upstroke, plateau) plus random flux sums."""
    rng = np.random.default_rng(seed)
    p = oracle.default_params()
    m = oracle.Model(p, 20, seed=seed)
    m.sample_initial_crus()
    m.set_globals(oracle.default_globals(py=True))
    istim = oracle.pulse_train(30000, 1e-3, 100.0, 0.5)
    out = []
    picks = set(np.linspace(0, 29999, n).astype(int).tolist())
    for i in range(30000):
        if i in picks:
            out.append(m.globals().to_array())
        m.euler_step(1e-3, istim[i])
    for g in out:
        yield g, rng


@pytest.mark.parametrize("over", [{}, {"Hf": 0.8, "Hr": 0.7}, {"GKr": 0.03, "PCaL": 1.1e-12, "Ko": 5.0}])
def test_global_step_matches_oracle(oracle, enginelib, over):
    from gwgb300 import _lib, engine

    p = oracle.default_params(**over)
    gp = engine.params_from({k: getattr(p, k) for k in _lib.PARAM_NAMES})
    n = 50
    worst = 0.0
    regimes = set()
    for g0, rng in _states(oracle, 3):
        regimes.add(bool(g0[0] >= -40.0))
        m = oracle.Model(p, n, seed=1)
        init = oracle.initial_crus(p, n, seed=2)
        init.ClCh[:] = rng.integers(0, 2, size=init.ClCh.shape)
        m.set_crus(init)
        m.set_globals(oracle.OrcGlobals.from_array(g0))
        JLCC = rng.uniform(-1e-3, 1e-3, size=(n, 4)) * (rng.random((n, 4)) < 0.3)
        Jxfer = rng.uniform(-1e-4, 1e-3, size=(n, 4))
        Jtr = rng.uniform(0, 5e-4, size=n)
        m.set_fluxes(JLCC, Jxfer, Jtr)
        Istim = float(rng.choice([0.0, 100.0]))
        m.euler_step(1e-3, Istim)
        ref = m.globals().to_array()
        sums = np.array([JLCC.sum(), float(init.ClCh.sum()), Jtr.sum(), Jxfer.sum()])
        g = g0.copy()
        sv = np.zeros(40)
        rc = enginelib.gw_global_step_host(C.byref(gp), n, g.ctypes.data_as(C.POINTER(C.c_double)),
                                           sums.ctypes.data_as(C.POINTER(C.c_double)), Istim, 1e-3,
                                           sv.ctypes.data_as(C.POINTER(C.c_double)))
        assert rc == 0
        # relative error of the increment (the state changes by ~1e-6 relative per step)
        dref, dgot = ref - g0, g - g0
        scale = np.maximum(np.abs(dref), 1e-12 * np.abs(g0) + 1e-300)
        worst = max(worst, float(np.max(np.abs(dgot - dref) / scale)))
        assert np.max(np.abs(g - ref) / np.maximum(np.abs(ref), 1e-300)) <= 1e-13
        # per-step SSA values at the new state against GW_model::SSA (GW.tpp:216-221)
        c = m.consts()
        c.VF_RT = float(ref[0]) * c.F_RT
        c.expmVF_RT = float(np.exp(-c.VF_RT))
        oracle.lib().orc_ssa_step_constants(C.byref(c), float(ref[0]))
        assert sv[4] == pytest.approx(c.alphaLCC, rel=1e-13)
        assert sv[5] == pytest.approx(c.betaLCC, rel=1e-13)
        assert sv[26] == pytest.approx(c.yinfLCC / c.tauLCC, rel=1e-13)
        assert sv[27] == pytest.approx((1.0 - c.yinfLCC) / c.tauLCC, rel=1e-13)
        assert sv[29] == pytest.approx(c.JLCC_exp, rel=1e-13)
        assert sv[28] == pytest.approx(c.JLCC_multiplier, rel=1e-12)
    assert regimes == {True, False}
    assert worst < 1e-9, worst
