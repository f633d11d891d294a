"""Post-processing (gwgb300.analysis) against the reference's own Python formulas (src/model.py),
where the reference sources are present: the currents from globals records, and ICaL, Ito2, Jtr,
Jxfer from record-time CRU sums against the same quantities summed from full CRU arrays."""
import sys

import numpy as np
import pytest

from gwgb300 import _lib, analysis


def _globals(rng, R):
    g = np.zeros((R, 36))
    names = _lib.GLOBAL_SCALARS
    g[:, names.index("V")] = rng.uniform(-90, 40, R)
    g[:, names.index("Nai")] = rng.uniform(8, 12, R)
    g[:, names.index("Ki")] = rng.uniform(125, 135, R)
    g[:, names.index("Cai")] = rng.uniform(1e-4, 1e-3, R)
    g[:, names.index("CaNSR")] = rng.uniform(0.5, 1.5, R)
    for n in ("m", "h", "j", "xKs", "CaLTRPN", "CaHTRPN"):
        g[:, names.index(n)] = rng.uniform(0.01, 0.99, R)
    g[:, 11:36] = rng.uniform(0.0, 0.2, (R, 25))
    return g


def test_currents_match_reference_python(ref_src):
    rng = np.random.default_rng(4)
    R = 64
    g = _globals(rng, R)
    p = ref_src.GWParameters(NCaRU_sim=100)
    m = ref_src.model
    names = _lib.GLOBAL_SCALARS
    G = lambda n: g[:, names.index(n)]  # noqa: E731
    V, Nai, Ki, Cai = G("V"), G("Nai"), G("Ki"), G("Cai")
    ours = analysis.currents(g, p)
    want = {"INa": m.INa(V, G("m"), G("h"), G("j"), Nai, p), "INab": m.INab(V, Nai, p),
            "IKr": m.IKr(V, g[:, 11 + 3], Ki, p), "IKs": m.IKs(V, G("xKs"), Ki, Nai, p),
            "IKv43": m.IKv43(V, g[:, 16 + 4], Ki, p), "IKv14": m.IKv14(V, g[:, 26 + 4], Ki, Nai, p),
            "IK1": m.IK1(V, Ki, p), "IKp": m.IKp(V, Ki, p), "INaK": m.INaK(V, Nai, p),
            "INaCa": m.INaCa(V, Nai, Cai, p), "IpCa": m.IpCa(Cai, p), "ICab": m.ICab(V, Cai, p),
            "Jup": m.Jup(Cai, G("CaNSR"), p)}
    for k, w in want.items():
        np.testing.assert_allclose(ours[k], w, rtol=1e-13, atol=0, err_msg=k)


def _cru_sums(LCC, LCCi, CaSS, RyR, ClCh, CaJSR):
    open_ = (LCC == 6) | (LCC == 12)
    cond = open_ & (LCCi == 1)
    n = LCC.shape[1]
    s = np.zeros((LCC.shape[0], 8))
    s[:, 0] = open_.sum(axis=(1, 2))
    s[:, 1] = cond.sum(axis=(1, 2))
    s[:, 2] = (CaSS * cond).sum(axis=(1, 2))
    s[:, 3] = (RyR[..., 2] + RyR[..., 3]).sum(axis=(1, 2))
    s[:, 4] = ClCh.sum(axis=(1, 2))
    s[:, 5] = CaSS.sum(axis=(1, 2))
    s[:, 6] = CaJSR.sum(axis=1)
    s[:, 7] = n
    return s


def test_cru_currents_from_sums_match_reference_python(ref_src):
    rng = np.random.default_rng(5)
    R, N = 7, 300
    g = _globals(rng, R)
    p = ref_src.GWParameters(NCaRU_sim=N)
    LCC = rng.integers(1, 13, (R, N, 4)).astype(np.int32)
    LCCi = rng.integers(0, 2, (R, N, 4)).astype(np.int32)
    ClCh = rng.integers(0, 2, (R, N, 4)).astype(np.int32)
    CaSS = rng.uniform(1e-4, 1e-2, (R, N, 4))
    CaJSR = rng.uniform(0.3, 1.2, (R, N))
    RyR = rng.integers(0, 3, (R, N, 4, 6)).astype(np.int32)
    s = _cru_sums(LCC, LCCi, CaSS, RyR, ClCh, CaJSR)
    ours = analysis.currents(g, p, cru_sums=s)
    V = g[:, 0]
    np.testing.assert_allclose(ours["ICaL"], ref_src.model.ICaL(V, LCC, LCCi, CaSS, p), rtol=1e-10)
    np.testing.assert_allclose(ours["Ito2"], ref_src.model.Ito2(V, ClCh, p), rtol=1e-10)
    # GWSolution.Jtr / Jxfer (model.py:885-899) sum over CRUs (and subunits) per record
    Cai, CaNSR = g[:, 3], g[:, 4]
    np.testing.assert_allclose(ours["Jtr"], p.rtr * (CaNSR[:, None] - CaJSR).sum(axis=1), rtol=1e-10)
    np.testing.assert_allclose(ours["Jxfer"], p.rxfer * (CaSS - Cai[:, None, None]).sum(axis=(1, 2)), rtol=1e-10)


def test_ap_markers():
    t = np.arange(1, 401) * 1.0
    V = np.full((2, 400), -90.0)
    V[0, 2:250] = 20.0
    V[1, 5:400] = 10.0  # does not repolarise in the window
    mk = analysis.ap_markers(t, V)
    assert mk["APD90"][0] == t[249] and mk["repolarised"].tolist() == [True, False]
    assert mk["APD90"][1] == t[-1] and mk["V_max"].tolist() == [20.0, 10.0]


def test_save_reduced_without_h5py(tmp_path, monkeypatch):
    from gwgb300.engine import Trace

    monkeypatch.setitem(sys.modules, "h5py", None)
    R, N = 3, 5
    rng = np.random.default_rng(6)
    tr = Trace(t=np.arange(R) * 0.5, globals=rng.uniform(size=(1, R, 36)),
               codec={"LCC": np.ones((R, N, 4), np.int8), "RyR": np.zeros((R, N, 4), np.int16),
                      "CaSS": np.zeros((R, N, 4), np.float32)})
    path = analysis.save_reduced(str(tmp_path / "run"), tr, _lib.default_params())
    z = np.load(path)
    assert z["vars/V"].dtype == np.float32 and z["vars/XKr"].shape == (R, 4) and z["vars/XKv14"].shape == (R, 9)
    assert z["vars/LCC"].dtype == np.int8 and z["vars/RyR"].dtype == np.int16
    assert float(z["params/GKr"]) == _lib.default_params().GKr
