"""Ensemble statistics of the FP32 engine against the FP64 engine (reference arithmetic, itself
checked bit-exact against the oracle): 200 replicate cells (one counter-RNG stream each), one
paced beat, two-sample Kolmogorov-Smirnov tests at alpha = 0.01 on the per-cell APD90 (censored
at the end of the 420 ms window, the same way for both), peak Cai, time of peak Cai and plateau
voltage.  With 200 CRUs per cell the beat-to-beat variability is large, which is what the
comparison of distributions needs."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N_CELLS = 200
NCRU = 200          # NCaRU stays 12,500: each simulated CRU stands for 62.5 (CRU_factor)
DT = 1e-3
T_MS = 420.0
EVERY = 500         # record every 0.5 ms
ALPHA = 0.01


def _ensemble_stats(precision, seed):
    from gwgb300 import Ensemble, _lib, engine

    e = Ensemble([NCRU] * N_CELLS, precision=precision, seed=seed)
    for c in range(N_CELLS):
        e.sample_initial_crus(c)
    e.set_pulse(0.0, 1000.0, 0.5, 100.0)
    tr = e.run(DT, int(T_MS / DT), record_every=EVERY)
    e.close()
    V = tr.var("V")      # [cells, records]
    Cai = tr.var("Cai")
    t = (np.arange(V.shape[1]) + 1) * EVERY * DT
    v_rest = engine.globals_to_array(_lib.default_globals(py=True))[0]
    v_max = V.max(axis=1)
    thr = v_rest + 0.1 * (v_max - v_rest)
    # APD90: last time above the 90 % repolarisation level (the beat starts at t = 0)
    above = V > thr[:, None]
    last = V.shape[1] - 1 - np.argmax(above[:, ::-1], axis=1)
    apd90 = t[last]
    i200 = int(round(200.0 / (EVERY * DT))) - 1
    return {"APD90": apd90, "peak_Cai": Cai.max(axis=1), "t_peak_Cai": t[Cai.argmax(axis=1)],
            "V_200ms": V[:, i200], "repolarised": V[:, -1] < -80.0, "V_max": v_max}


@pytest.fixture(scope="module")
def stats():
    return _ensemble_stats("fp32", seed=101), _ensemble_stats("fp64", seed=202)


def test_every_cell_fires_and_most_repolarise(stats):
    s32, s64 = stats
    for s in (s32, s64):
        assert np.all(s["V_max"] > 20.0) and np.all(s["peak_Cai"] > 2e-4)
        assert s["repolarised"].mean() > 0.5
    # the fraction repolarised by the end of the window agrees (binomial standard error ~0.03)
    assert abs(s32["repolarised"].mean() - s64["repolarised"].mean()) < 0.15


@pytest.mark.parametrize("name", ["APD90", "peak_Cai", "t_peak_Cai", "V_200ms"])
def test_fp32_matches_fp64_distribution(stats, name):
    from scipy.stats import ks_2samp

    s32, s64 = stats
    a, b = s32[name], s64[name]
    r = ks_2samp(a, b)
    assert r.pvalue > ALPHA, (name, r.statistic, r.pvalue, float(np.mean(a)), float(np.mean(b)))
