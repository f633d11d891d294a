"""Record-time outputs written by the device: the per-cell CRU sums (gw_trace.cru_sums) and the
reduced-memory CRU records (gw_trace codec arrays), against the full CRU records of an identical
run (same seed, so the same trajectory): counts exact, Ca sums within their 2^-40 mM resolution,
codec arrays equal to the conversions of the reference's serialization (utils.py:8-22)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NCRU = [700, 520]
EVERY = 100
STEPS = 1500


def _ens(precision):
    from gwgb300 import Ensemble

    e = Ensemble(NCRU, precision=precision, seed=13)
    for c in range(len(NCRU)):
        e.sample_initial_crus(c)
    e.set_pulse(0.0, 1000.0, 0.5, 100.0)
    return e


def _sums_from_arrays(cr):
    LCC, LCCi, CaSS, RyR, ClCh, CaJSR = (cr[k] for k in ("LCC", "LCC_inactivation", "CaSS", "RyR", "ClCh", "CaJSR"))
    open_ = (LCC == 6) | (LCC == 12)
    cond = open_ & (LCCi == 1)
    s = np.zeros((LCC.shape[0], 8))
    s[:, 0] = open_.sum(axis=(1, 2))
    s[:, 1] = cond.sum(axis=(1, 2))
    s[:, 2] = (CaSS * cond).sum(axis=(1, 2))
    s[:, 3] = (RyR[..., 2] + RyR[..., 3]).sum(axis=(1, 2))
    s[:, 4] = ClCh.sum(axis=(1, 2))
    s[:, 5] = CaSS.sum(axis=(1, 2))
    s[:, 6] = CaJSR.sum(axis=1)
    s[:, 7] = LCC.shape[1]
    return s


def _ryr_code(RyR):
    """The reference's RyR_state_to_int16 (utils.py:8-22), restated."""
    r = RyR.astype(np.int64)
    neg34 = (r[..., 2] < 0) | (r[..., 3] < 0)
    q2 = np.where(neg34, r[..., 2] + r[..., 3], r[..., 2])
    q3 = np.where(neg34, 0, r[..., 3])
    neg56 = (r[..., 4] < 0) | (r[..., 5] < 0)
    q4 = np.where(neg56, r[..., 4] + r[..., 5], r[..., 4])
    return (r[..., 0] + 6 * r[..., 1] + 36 * q2 + 216 * q3 + 1296 * q4).astype(np.int16)


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_sums_and_codec_match_full_records(precision):
    a, b = _ens(precision), _ens(precision)
    ta = a.run(1e-3, STEPS, record_every=EVERY, cru_cell=1, sums=True)
    tb = b.run(1e-3, STEPS, record_every=EVERY, cru_cell=1, sums=True, codec=True)
    a.close()
    b.close()
    R = STEPS // EVERY
    assert ta.cru_sums.shape == (2, R, 8) and tb.codec["LCC"].shape == (R, NCRU[1], 4)
    # same trajectory, and the sums do not depend on the record format or on timing
    np.testing.assert_array_equal(ta.globals, tb.globals)
    np.testing.assert_array_equal(ta.cru_sums, tb.cru_sums)
    # sums of cell 1 against its full records
    want = _sums_from_arrays(ta.crus)
    got = ta.cru_sums[1]
    for f in (0, 1, 3, 4, 7):
        np.testing.assert_array_equal(got[:, f], want[:, f])
    n = NCRU[1]
    for f, terms in ((2, 4 * n), (5, 4 * n), (6, 2 * n)):
        tol = terms * 2.0 ** -40 + 1e-13 * np.abs(want[:, f])
        if f == 6 and precision == "fp32":
            tol = tol + n * 2.0 ** -24  # the device sums CaJSR with its compensation term, the record holds the float
        assert np.all(np.abs(got[:, f] - want[:, f]) <= tol), f
    assert np.all(ta.cru_sums[0][:, 7] == NCRU[0]) and np.all(ta.cru_sums[0][:, 5] > 0)
    assert want[:, 0].max() > 0  # the records cover open LCCs (the AP)
    # codec against the full records
    cr, cd = ta.crus, tb.codec
    np.testing.assert_array_equal(cd["LCC"], cr["LCC"].astype(np.int8))
    np.testing.assert_array_equal(cd["LCC_inactivation"], cr["LCC_inactivation"].astype(np.bool_))
    np.testing.assert_array_equal(cd["ClCh"], cr["ClCh"].astype(np.bool_))
    np.testing.assert_array_equal(cd["RyR"], _ryr_code(cr["RyR"]))
    np.testing.assert_array_equal(cd["CaSS"], cr["CaSS"].astype(np.float32))
    np.testing.assert_array_equal(cd["CaJSR"], cr["CaJSR"].astype(np.float32))


def test_currents_from_device_sums():
    from gwgb300 import _lib, analysis

    e = _ens("fp32")
    tr = e.run(1e-3, STEPS, record_every=EVERY, cru_cell=0, sums=True)
    e.close()
    p = _lib.default_params()
    c_sums = analysis.currents(tr.globals[0], p, cru_sums=tr.cru_sums[0])
    c_full = analysis.currents(tr.globals[0], p, cru_sums=_sums_from_arrays(tr.crus))
    for k in ("ICaL", "Ito2", "Jxfer", "LCC_open_fraction", "RyR_open_fraction"):
        np.testing.assert_allclose(c_sums[k], c_full[k], rtol=1e-9, atol=1e-12, err_msg=k)
    # Jtr: the device's CaJSR sum carries the compensation term the float records do not
    np.testing.assert_allclose(c_sums["Jtr"], c_full["Jtr"], rtol=1e-9, atol=p.rtr * NCRU[0] * 2.0 ** -23)
    assert np.all(c_sums["ICaL"] <= 0)  # inward


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_currents_on_device_match_host_formulas(precision):
    """gw_trace.currents (the reference's GWSolution currents evaluated by the device at every record
    of every cell) against gwgb300.analysis.currents (the same formulas on the host, checked against
    the reference's own Python in tests/test_analysis.py) on the same records, for two cells with
    their own parameters and CRU counts, over the upstroke and Ca release."""
    from gwgb300 import Ensemble, _lib, analysis, engine

    d = _lib.default_params()
    params = [engine.params_from(None, GKr=d.GKr * 1.2, PCaL=d.PCaL * 0.8, NCaRU=7000),
              engine.params_from(None, GK1=d.GK1 * 0.9, Vmaxf=d.Vmaxf * 1.1, Vmaxr=d.Vmaxr * 1.1, NCaRU=12500)]
    e = Ensemble(NCRU, params, precision=precision, seed=17)
    for c in range(len(NCRU)):
        e.sample_initial_crus(c)
    e.set_pulse(0.0, 1000.0, 0.5, 100.0)
    tr = e.run(1e-3, 30_000, record_every=250, sums=True, currents=True)
    e.close()
    R = 30_000 // 250
    assert tr.currents.shape == (2, R, len(_lib.CURRENT_FIELDS))
    for c in range(2):
        host = analysis.currents(tr.globals[c], params[c], cru_sums=tr.cru_sums[c])
        for k, name in enumerate(_lib.CURRENT_FIELDS):
            dev, ref = tr.currents[c, :, k], host[name]
            scale = max(float(np.max(np.abs(ref))), 1e-300)
            np.testing.assert_allclose(dev, ref, rtol=1e-10, atol=1e-12 * scale, err_msg=f"cell {c} {name}")
    assert tr.current("ICaL").min() < 0 and tr.var("V").max() > 0  # an upstroke with an inward ICaL


def test_noalloc_rejects_sums_and_codec():
    import ctypes as C

    from gwgb300 import _lib

    e = _ens("fp32")
    tr = _lib.GwTrace()
    tr.max_records = 2
    s = np.zeros((2, 2, 8))
    tr.cru_sums = s.ctypes.data_as(C.POINTER(C.c_double))
    assert e.L.gw_run_noalloc(e.h, 1e-3, 20, 10, C.byref(tr)) == _lib.GW_ERR_INVALID_ARGUMENT
    tr.cru_sums = None
    cur = np.zeros((2, 2, len(_lib.CURRENT_FIELDS)))
    tr.currents = cur.ctypes.data_as(C.POINTER(C.c_double))
    assert e.L.gw_run_noalloc(e.h, 1e-3, 20, 10, C.byref(tr)) == _lib.GW_ERR_INVALID_ARGUMENT
    e.close()
