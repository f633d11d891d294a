"""Post-processing of recorded traces: the currents of the reference's GWSolution, action-potential
markers, and the reduced-memory trace file.

`currents` evaluates the reference's Python current formulas (src/model.py:46-549, GWSolution
properties :771-899) vectorised over [cells, records].  The CRU-dependent ones (ICaL, Ito2, Jtr,
Jxfer) come from the record-time CRU sums that the device reduces (Trace.cru_sums), so the CRU
arrays never leave the device; the rest come from the recorded globals.  Note that these are the
reference's Python formulas, which differ from its C++ step in places (ICaL uses exp(2VF/RT)).
"""
from __future__ import annotations

from typing import Dict, Optional

import numpy as np

from . import _lib

F = 96.5        # model.py:14-16
R_GAS = 8.314
F_R = F / R_GAS

_G = {n: i for i, n in enumerate(_lib.GLOBAL_SCALARS)}
_KR, _KV43, _KV14 = 11, 16, 26   # offsets of XKr, XKv43, XKv14 in a globals record


def _par(params, name):
    return float(getattr(params, name))


def reversal_potentials(g: np.ndarray, params) -> Dict[str, np.ndarray]:
    """ENa, EK, EKs, ECa (model.py:46-117) of globals records g[..., 36]."""
    F_RT = F_R / _par(params, "T")
    Nai, Ki, Cai = g[..., _G["Nai"]], g[..., _G["Ki"]], g[..., _G["Cai"]]
    Nao, Ko, Cao = _par(params, "Nao"), _par(params, "Ko"), _par(params, "Cao")
    return {"ENa": np.log(Nao / Nai) / F_RT, "EK": np.log(Ko / Ki) / F_RT,
            "EKs": np.log((Ko + 0.01833 * Nao) / (Ki + 0.01833 * Nai)) / F_RT,
            "ECa": 0.5 * np.log(Cao / Cai) / F_RT}


def currents(g: np.ndarray, params, ncru=None, cru_sums: Optional[np.ndarray] = None) -> Dict[str, np.ndarray]:
    """The reference's currents [pA/pF] and fluxes [mM/ms] for globals records g[..., 36]; with
    cru_sums[..., 8] also ICaL, Ito2, Jtr, Jxfer and the LCC / RyR open fractions (the simulated
    CRU count is the sums' CRUs field unless ncru is given)."""
    P = lambda n: _par(params, n)  # noqa: E731
    T = P("T")
    V = g[..., _G["V"]]
    Nai, Ki, Cai, CaNSR = g[..., _G["Nai"]], g[..., _G["Ki"]], g[..., _G["Cai"]], g[..., _G["CaNSR"]]
    m, h, j, xKs = g[..., _G["m"]], g[..., _G["h"]], g[..., _G["j"]], g[..., _G["xKs"]]
    XKr = g[..., _KR + 3]
    XKv43 = g[..., _KV43 + 4]
    XKv14 = g[..., _KV14 + 4]
    E = reversal_potentials(g, params)
    Ko, Nao, Cao = P("Ko"), P("Nao"), P("Cao")
    out = {}
    out["INa"] = P("GNa") * (m ** 3) * h * j * (V - E["ENa"])
    out["INab"] = P("GNab") * (V - E["ENa"])
    RKr = 1 / (1 + 1.4945 * np.exp(0.0446 * V))
    out["IKr"] = 0.5 * P("GKr") * np.sqrt(Ko) * RKr * XKr * (V - E["EK"])
    out["IKs"] = P("GKs") * (xKs ** 2) * (V - E["EKs"])
    out["IKv43"] = P("GKv43") * XKv43 * (V - E["EK"])
    VF_RT = V * F_R / T
    eVF = np.exp(VF_RT)
    mult14 = (P("PKv14") / P("Csc")) * F * VF_RT * XKv14 / (1 - eVF)
    out["IKv14"] = mult14 * ((Ki - Ko * eVF) + 0.02 * (Nai - Nao)) * 1e9
    out["Ito1"] = out["IKv14"] + out["IKv43"]
    K1inf = 1 / (2 + np.exp(1.5 * (V - E["EK"]) * F_R / T))
    out["IK1"] = P("GK1") * K1inf * (Ko / (Ko + P("KmK1"))) * (V - E["EK"])
    Kp = 1 / (1 + np.exp((7.488 - V) / 5.98))
    out["IKp"] = P("GKp") * Kp * (V - E["EK"])
    sigma = (np.exp(Nao / 67.3) - 1) / 7
    fNaK = 1 / (1 + 0.1245 * np.exp(-0.1 * V * F_R / T) + 0.0365 * sigma * np.exp(-V * F_R / T))
    multNaK = P("INaKmax") * Ko / (Ko + P("KmKo"))
    out["INaK"] = multNaK * fNaK / (1 + (P("KmNai") / Nai) ** 1.5)
    e1 = np.exp(P("eta") * V * F_R / T)
    e2 = np.exp((P("eta") - 1) * V * F_R / T)
    multNaCa = 5000 * P("kNaCa") / ((P("KmNa") ** 3 + Nao ** 3) * (P("KmCa") + Cao))
    out["INaCa"] = multNaCa * (e1 * (Nai ** 3) * Cao - e2 * (Nao ** 3) * Cai) / (1 + P("ksat") * e2)
    out["IpCa"] = P("IpCamax") * (Cai / (P("KmpCa") + Cai))
    out["ICab"] = P("GCab") * (V - E["ECa"])
    f = (Cai / P("Kmf")) ** P("Hf")
    r = (CaNSR / P("Kmr")) ** P("Hr")
    out["Jup"] = (P("Vmaxf") * f - P("Vmaxr") * r) / (1 + f + r)
    if cru_sums is not None:
        S = lambda k: cru_sums[..., _lib.SUM_FIELDS.index(k)]  # noqa: E731
        scale = P("NCaRU") / (S("CRUs") if ncru is None else np.asarray(ncru, dtype=float))  # NCaRU / NCaRU_sim
        e2VF = np.exp(2 * VF_RT)
        multL = scale * (P("PCaL") / P("CSA")) * (4 * F * VF_RT) / (e2VF - 1)
        out["ICaL"] = multL * (e2VF * S("CaSS_conducting") - 0.341 * Cao * S("LCC_conducting")) * 1e9
        emVF = np.exp(-VF_RT)
        multT = scale * (P("Pto2") / P("CSA")) * (F * VF_RT) / (emVF - 1)
        out["Ito2"] = multT * S("ClCh_open") * (P("Clcyto") * emVF - P("Clo")) * 1e9
        out["Jtr"] = P("rtr") * (S("CRUs") * CaNSR - S("CaJSR"))
        out["Jxfer"] = P("rxfer") * (S("CaSS") - 4 * S("CRUs") * Cai)
        out["LCC_open_fraction"] = S("LCC_open") / (4 * S("CRUs"))
        out["RyR_open_fraction"] = S("RyR_open") / (20 * S("CRUs"))
    return out


def ap_markers(t: np.ndarray, V: np.ndarray, v_rest: Optional[float] = None) -> Dict[str, np.ndarray]:
    """Per trace (last axis = records): peak V, its time, and APD90 = the last time V is above
    v_rest + 0.1 (V_max - v_rest) (the window end if it never repolarises)."""
    V = np.asarray(V)
    vr = V[..., 0] if v_rest is None else np.full(V.shape[:-1], float(v_rest))
    vmax = V.max(axis=-1)
    thr = vr + 0.1 * (vmax - vr)
    above = V > thr[..., None]
    last = V.shape[-1] - 1 - np.argmax(above[..., ::-1], axis=-1)
    return {"V_max": vmax, "t_V_max": np.asarray(t)[V.argmax(axis=-1)], "APD90": np.asarray(t)[last],
            "repolarised": V[..., -1] < thr}


def reduced_memory_vars(trace, cell: int = 0) -> Dict[str, np.ndarray]:
    """The variables of the reference's reduced-memory trace (serialization.py:11-39) for one
    cell: float32 globals (XKr without state 5, XKv14/XKv43 without state 10) and, when the trace
    holds them, the device-written CRU codec arrays."""
    g = np.asarray(trace.globals[cell])
    out = {"t": np.float32(trace.t)}
    for n in _lib.GLOBAL_SCALARS:
        out[n] = np.float32(g[:, _G[n]])
    out["XKr"] = np.float32(g[:, _KR:_KR + 4])
    out["XKv14"] = np.float32(g[:, _KV14:_KV14 + 9])
    out["XKv43"] = np.float32(g[:, _KV43:_KV43 + 9])
    if trace.codec is not None:
        for k, v in trace.codec.items():
            out[k] = v
    return out


def save_reduced(path: str, trace, params, cell: int = 0) -> str:
    """Writes the reduced-memory trace: HDF5 with groups params / vars (gzip) when h5py is
    installed, as the reference's save_sim (serialization.py:42-53) does; otherwise a compressed
    .npz with keys params/<name> and vars/<name>.  Returns the path written."""
    vars_ = reduced_memory_vars(trace, cell)
    pars = {n: getattr(params, n) for n, _ in type(params)._fields_} if hasattr(type(params), "_fields_") else dict(params)
    try:
        import h5py  # noqa: F401
    except ImportError:
        h5py = None
    if h5py is not None:
        with h5py.File(path, "w") as f:
            pg = f.create_group("params")
            for k, v in pars.items():
                pg.create_dataset(name=k, data=v)
            vg = f.create_group("vars")
            for k, v in vars_.items():
                vg.create_dataset(name=k, data=v, compression="gzip")
        return path
    if not path.endswith(".npz"):
        path = path + ".npz"
    np.savez_compressed(path, **{f"params/{k}": np.asarray(v) for k, v in pars.items()},
                        **{f"vars/{k}": v for k, v in vars_.items()})
    return path
