"""Parity of a heterogeneous ensemble (the batched form) with per-cell oracle runs, FP64.

One engine context holds cells of uneven CRU counts (5 ... 1,200), each with its own parameter
set (PCaL, GKr, GKs, Vmaxf = Vmaxr and rRyR scaled by log-normal(sigma = 0.1) factors, as the
reference's Constants ctor derives them per cell, src/includes/GW_utils.tpp:67-116), its own
NCaRU, and its own pacing cycle length (400-1000 ms, pulse train evaluated on the device); the
launch shape is the autotuner's.  The run covers a full beat of the shortest cycle lengths (410 ms:
the cells paced at 400 and 405 ms get their second stimulus).  Each cell must equal the oracle run
of that cell alone, keyed by its cell index:

  channel states   bit-exact (final state, and the trace cell's CRU arrays at every record)
  CaSS, CaJSR      within 1e-12 relative
  globals          within 1e-12 relative, at every record of every cell
"""
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CHANNELS = ("LCC", "LCC_inactivation", "RyR", "ClCh")
DT = 1e-3


def rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300))) if a.size else 0.0


def ensemble_case(seed=2024):
    rng = np.random.default_rng(seed)
    ncru = [17, 1200, 64, 333, 5, 700, 250, 960]
    ncaru = [170, 12500, 640, 12500, 50, 12500, 2500, 12500]
    cl = [400.0, 1000.0, 415.0, 650.0, 480.0, 820.0, 405.0, 560.0]
    scale = rng.lognormal(0.0, 0.1, size=(len(ncru), 5))
    return ncru, ncaru, cl, scale


def cell_params(po, ncaru, f):
    d = po.default_params()
    return po.default_params(PCaL=d.PCaL * f[0], GKr=d.GKr * f[1], GKs=d.GKs * f[2], Vmaxf=d.Vmaxf * f[3],
                             Vmaxr=d.Vmaxr * f[3], rRyR=d.rRyR * f[4], NCaRU=int(ncaru))


def test_heterogeneous_ensemble_matches_per_cell_oracle(oracle):
    from gwgb300 import Ensemble, engine

    po = oracle
    seed, steps, every, trace_cell = 77, 410_000, 5000, 1
    ncru, ncaru, cl, scale = ensemble_case()
    params = [cell_params(po, ncaru[c], scale[c]) for c in range(len(ncru))]
    e = Ensemble(ncru, [engine.params_from(p) for p in params], precision="fp64", seed=seed,
                 cluster_ctas="auto", tune_steps=100)
    for c in range(len(ncru)):
        e.sample_initial_crus(c)
        e.set_pulse(0.0, cl[c], 0.5, 100.0, cell=c)
    tr = e.run(DT, steps, record_every=every, cru_cell=trace_cell)
    shape = e.stats()
    finals = [(e.get_globals(c), e.get_crus(c)) for c in range(len(ncru))]
    e.close()

    cores = os.cpu_count() or 1
    total = float(sum(ncru))

    def oracle_cell(c):
        po.lib().orc_set_threads(max(1, int(round(cores * ncru[c] / total))))
        m = po.Model(params[c], ncru[c], seed=seed, cell=c)
        m.sample_initial_crus()
        made, rec = m.run_record(DT, po.pulse_train(steps, DT, 100.0, 0.5, cl[c]), every)
        return m.globals().to_array(), m.crus(), rec

    with ThreadPoolExecutor(max_workers=len(ncru)) as ex:
        ref = list(ex.map(oracle_cell, range(len(ncru))))

    assert shape["cluster_ctas"] >= 1
    np.testing.assert_array_equal(tr.t, ref[0][2]["t"])
    for c, ((g, s), (g_ref, s_ref, rec)) in enumerate(zip(finals, ref)):
        for k in CHANNELS:
            np.testing.assert_array_equal(getattr(s, k), getattr(s_ref, k), err_msg=f"cell {c} {k}")
        assert rel(s.CaSS, s_ref.CaSS) <= 1e-12, c
        assert rel(s.CaJSR, s_ref.CaJSR) <= 1e-12, c
        assert rel(g, g_ref) <= 1e-12, c
        assert rel(tr.globals[c], rec["globals"]) <= 1e-12, c
    rec = ref[trace_cell][2]
    for k in CHANNELS:
        np.testing.assert_array_equal(tr.crus[k], rec[k], err_msg=k)
    assert rel(tr.crus["CaSS"], rec["CaSS"]) <= 1e-12
    # the cell paced at 400 ms was stimulated a second time: records after steps 395,000 and
    # 405,000 lie either side of its second upstroke
    V0 = tr.globals[0, :, 0]
    assert V0[405_000 // every] - V0[395_000 // every] > 30.0, V0[-4:]


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_partition_contexts_reproduce_one_context(oracle, precision):
    """The ensemble split into contiguous shares (Ensemble.partitioned: cell_base = the share's first
    global cell, the whole ensemble's launch shape), one context per share as one rank per GPU
    would hold them, gives the one-context results bit for bit: globals at every record, final
    CRU arrays including JLCC, and the flux carries."""
    from gwgb300 import Ensemble, engine

    po = oracle
    seed, steps, every = 5, 3000, 500
    ncru, ncaru, cl, scale = ensemble_case()
    params = [engine.params_from(cell_params(po, ncaru[c], scale[c])) for c in range(len(ncru))]

    def run(e, cells):
        for i, c in enumerate(cells):
            e.sample_initial_crus(i)
            e.set_pulse(0.0, cl[c], 0.5, 100.0, cell=i)
        tr = e.run(DT, steps, record_every=every)
        crus = [e.get_crus(i) for i in range(len(cells))]
        carry = [e.get_flux_carry(i) for i in range(len(cells))]
        return tr.globals, crus, carry

    whole = Ensemble(ncru, params, precision=precision, seed=seed)
    Gw, Cw, Fw = run(whole, range(len(ncru)))
    whole.close()
    for world in (2, 3):
        got_G, got_C, got_F = [], [], []
        for rank in range(world):
            part = Ensemble.partitioned(ncru, params, world=world, rank=rank, precision=precision, seed=seed)
            cells = list(part.global_cells)
            G, Cr, F = run(part, cells)
            part.close()
            got_G.append(G)
            got_C += Cr
            got_F += F
        np.testing.assert_array_equal(np.concatenate(got_G, axis=0), Gw)
        for c in range(len(ncru)):
            for k in ("CaSS", "CaJSR", "JLCC") + CHANNELS:
                np.testing.assert_array_equal(getattr(got_C[c], k), getattr(Cw[c], k), err_msg=f"{world} {c} {k}")
            assert got_F[c] == Fw[c]
