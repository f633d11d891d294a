"""Drop-in for the reference's pybind11 module ``GreensteinWinslow`` (src/pyGW.cpp:160-344).

src/model.py and src/parameters.py import it as ``build.GreensteinWinslow``.  The classes and
``run`` keep the reference's names, fields, argument order and errors; ``run`` simulates on the GB300
engine through the C ABI (gw_simulate).

Differences a caller can see:
- ``Istim`` (a callable) is evaluated on the host once per step at t_i = sum_{k<i} step_size before
  the run, as the reference's loop would evaluate it (pyGW.hpp:110-116); a NumPy array of per-step
  values is accepted as well.
- The PRNG name is validated as in the reference (unknown names raise ValueError) but draws come from
  the engine's counter-based stream; ``seed`` (keyword) fixes it, otherwise a fresh seed is drawn.
- ``precision`` (keyword): "fp64" (default, reference arithmetic) or "fp32".
- ``GWCRUState(N)`` starts from the reference's random initial distributions (GW_utils.tpp:5-64)
  instead of uninitialised memory.
- The reference allocates num_steps // record_every records but writes one more when record_every
  does not divide num_steps (pyGW.hpp:109,117-119); this module keeps the first num_steps //
  record_every records.
"""
from __future__ import annotations

import ctypes as C
import os
import secrets

import numpy as np

from gwgb300 import _lib
from gwgb300._lib import GwGlobals, GwParams, GwTrace, check

_PRNGS = ("mt19937", "mt19937_64", "xoshiro256+", "xoshiro256++", "xoshiro256**", "xoroshiro128+",
          "xoroshiro128++", "xoroshiro128**")


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


class GWParameters:
    """GW::Parameters with read/write fields (pyGW.cpp:168-285)."""

    def __init__(self):
        p = GwParams()
        _lib.load(build_if_missing=True).gw_params_default(C.byref(p))
        for n in _lib.PARAM_NAMES:
            object.__setattr__(self, n, getattr(p, n))

    def __setattr__(self, name, value):
        if name not in _lib.PARAM_NAMES:
            raise AttributeError(f"'GWParameters' object has no attribute '{name}'")
        object.__setattr__(self, name, int(value) if name == "NCaRU" else float(value))

    def __repr__(self):
        return "Greenstein and Winslow Model Parameters"

    def _struct(self) -> GwParams:
        p = GwParams()
        for n in _lib.PARAM_NAMES:
            setattr(p, n, getattr(self, n))
        return p


def _arr(value, dtype, shape=None):
    a = np.array(value, dtype=dtype, copy=True)
    if shape is not None and a.shape != shape:
        a = a.reshape(shape)
    return a


class GWGlobalState:
    """Initial global state (pyGW.cpp:31-76)."""

    _SCALARS = _lib.GLOBAL_SCALARS

    def __init__(self):
        g = GwGlobals()
        _lib.load().gw_globals_py_default(C.byref(g))
        for n in self._SCALARS:
            object.__setattr__(self, n, float(getattr(g, n)))
        object.__setattr__(self, "XKr", np.array(list(g.Kr), dtype=np.float64))
        object.__setattr__(self, "XKv14", np.array(list(g.Kv14), dtype=np.float64))
        object.__setattr__(self, "XKv43", np.array(list(g.Kv43), dtype=np.float64))

    def __setattr__(self, name, value):
        if name in self._SCALARS:
            object.__setattr__(self, name, float(value))
        elif name == "XKr":
            object.__setattr__(self, name, _arr(value, np.float64, (5,)))
        elif name in ("XKv14", "XKv43"):
            object.__setattr__(self, name, _arr(value, np.float64, (10,)))
        else:
            raise AttributeError(f"'GWGlobalState' object has no attribute '{name}'")

    def _struct(self) -> GwGlobals:
        g = GwGlobals()
        for n in self._SCALARS:
            setattr(g, n, getattr(self, n))
        for i in range(5):
            g.Kr[i] = self.XKr[i]
        for i in range(10):
            g.Kv14[i] = self.XKv14[i]
            g.Kv43[i] = self.XKv43[i]
        return g


def _initial_cru_arrays(n: int, rng: np.random.Generator):
    """The reference's random initial CRU distributions (GW_utils.tpp:5-64)."""
    LCC = rng.choice(np.array([1, 2, 7], dtype=np.int32), p=[0.958, 0.038, 0.004], size=(n, 4))
    LCCi = (rng.random((n, 4)) < 0.9425).astype(np.int32)
    ClCh = (rng.random((n, 4)) < 0.002).astype(np.int32)
    RyR = np.zeros((n, 4, 6), dtype=np.int32)
    pick = rng.choice(np.array([0, 4, 5]), p=[0.609, 0.5 * 0.391, 0.5 * 0.391], size=(n, 4, 5))
    for k in (0, 4, 5):
        RyR[..., k] = (pick == k).sum(axis=-1)
    return LCC.astype(np.int32), LCCi, RyR, ClCh


class GWCRUState:
    """Initial CRU state (pyGW.cpp:78-87)."""

    _SHAPES = {"CaSS": ((4,), np.float64), "CaJSR": ((), np.float64), "LCC": ((4,), np.int32),
               "LCC_inactivation": ((4,), np.int32), "RyR": ((4, 6), np.int32),
               "ClCh": ((4,), np.int32)}

    def __init__(self, nCRU: int):
        n = int(nCRU)
        object.__setattr__(self, "_n", n)
        LCC, LCCi, RyR, ClCh = _initial_cru_arrays(n, np.random.default_rng(0))
        object.__setattr__(self, "CaSS", np.full((n, 4), 1.45370e-4))
        object.__setattr__(self, "CaJSR", np.full(n, 0.908408))
        object.__setattr__(self, "LCC", LCC)
        object.__setattr__(self, "LCC_inactivation", LCCi)
        object.__setattr__(self, "RyR", RyR)
        object.__setattr__(self, "ClCh", ClCh)

    def __setattr__(self, name, value):
        if name not in self._SHAPES:
            raise AttributeError(f"'GWCRUState' object has no attribute '{name}'")
        tail, dt = self._SHAPES[name]
        a = np.array(value, dtype=dt, copy=True)
        if a.shape[1:] != tail:
            raise ValueError(f"{name} must have shape (N, {', '.join(map(str, tail))})")
        object.__setattr__(self, name, a)


class GWVariables:
    """Recorded solution (PyGWSimulation, pyGW.hpp:22-53; fields pyGW.cpp:288-311)."""

    _FIELDS = {"t": ((), np.float64), "V": ((), np.float64), "m": ((), np.float64),
               "h": ((), np.float64), "j": ((), np.float64), "Nai": ((), np.float64),
               "Ki": ((), np.float64), "Cai": ((), np.float64), "CaNSR": ((), np.float64),
               "CaLTRPN": ((), np.float64), "CaHTRPN": ((), np.float64), "xKs": ((), np.float64),
               "XKr": ((5,), np.float64), "XKv14": ((10,), np.float64), "XKv43": ((10,), np.float64),
               "CaJSR": (("n",), np.float64), "CaSS": (("n", 4), np.float64),
               "LCC": (("n", 4), np.int32), "LCC_inactivation": (("n", 4), np.int32),
               "RyR": (("n", 4, 6), np.int32), "ClCh": (("n", 4), np.int32)}

    def __init__(self, nCRU: int, num_step: int, t: float):
        object.__setattr__(self, "nCRU", int(nCRU))
        object.__setattr__(self, "tspan", float(t))
        R = int(num_step)
        for name, (tail, dt) in self._FIELDS.items():
            shape = (R,) + tuple(self.nCRU if d == "n" else d for d in tail)
            object.__setattr__(self, name, np.zeros(shape, dtype=dt))

    def __setattr__(self, name, value):
        if name not in self._FIELDS:
            raise AttributeError(f"'GWVariables' object has no attribute '{name}'")
        object.__setattr__(self, name, np.array(value, dtype=self._FIELDS[name][1], copy=True))

    def __repr__(self):
        return ("Greenstein and Winslow model solution over the interval [0, %f] with %d CRUs"
                % (self.tspan, self.nCRU))


def run(parameters, nCRU, step_size, num_steps, Istim, record_every, init_crus,
        init_globals=None, PRNG="mt19937_64", *, seed=None, precision="fp64"):
    """Simulate the model (pyGW.cpp:341-344 -> run_PRNG_arg, pyGW.cpp:134-157)."""
    if PRNG not in _PRNGS:
        raise ValueError(str(PRNG))
    if init_globals is None:
        init_globals = GWGlobalState()
    nCRU = int(nCRU)
    num_steps = int(num_steps)
    record_every = int(record_every)
    step_size = float(step_size)
    if nCRU <= 0 or num_steps < 0 or record_every <= 0:
        raise ValueError("nCRU and record_every must be > 0 and num_steps >= 0")
    if precision not in _lib.PRECISION:
        raise ValueError(f"precision must be one of {list(_lib.PRECISION)}")
    L = _lib.load()
    if callable(Istim):
        samples = np.empty(num_steps, dtype=np.float64)
        t = 0.0
        for i in range(num_steps):
            samples[i] = Istim(t)
            t += step_size
    else:
        samples = np.ascontiguousarray(Istim, dtype=np.float64)
        if samples.size != num_steps:
            raise ValueError("Istim samples must have num_steps values")
    def crus(name, dt, shape):
        a = np.ascontiguousarray(getattr(init_crus, name), dtype=dt)
        if a.shape != shape:
            raise ValueError(f"init_crus.{name} has shape {a.shape}, expected {shape}")
        return a
    CaSS = crus("CaSS", np.float64, (nCRU, 4))
    CaJSR = crus("CaJSR", np.float64, (nCRU,))
    LCC = crus("LCC", np.int32, (nCRU, 4))
    LCCi = crus("LCC_inactivation", np.int32, (nCRU, 4))
    RyR = crus("RyR", np.int32, (nCRU, 4, 6))
    ClCh = crus("ClCh", np.int32, (nCRU, 4))
    nrec = num_steps // record_every
    out = GWVariables(nCRU, nrec, num_steps * step_size)
    G = np.zeros((max(nrec, 1), 36))
    tr = GwTrace()
    tr.max_records = nrec
    tr.t = _dp(out.t)
    tr.globals = _dp(G)
    tr.cru_cell = 0
    tr.CaSS, tr.CaJSR = _dp(out.CaSS), _dp(out.CaJSR)
    tr.LCC, tr.LCC_inactivation = _ip(out.LCC), _ip(out.LCC_inactivation)
    tr.RyR, tr.ClCh = _ip(out.RyR), _ip(out.ClCh)
    if seed is None:
        seed = secrets.randbits(64)
    g = init_globals._struct() if hasattr(init_globals, "_struct") else _globals_struct(init_globals)
    p = parameters._struct() if hasattr(parameters, "_struct") else _params_struct(parameters)
    rc = L.gw_simulate(C.byref(p), nCRU, step_size, num_steps, _dp(samples), record_every, _dp(CaSS),
                       _dp(CaJSR), _ip(LCC), _ip(LCCi), _ip(RyR), _ip(ClCh), C.byref(g),
                       PRNG.encode(), int(seed) & 0xFFFFFFFFFFFFFFFF, _lib.PRECISION[precision],
                       C.byref(tr))
    check(rc)
    k = nrec
    Gk = G[:k]
    for i, n in enumerate(_lib.GLOBAL_SCALARS):
        object.__setattr__(out, n, Gk[:, i].copy())
    object.__setattr__(out, "XKr", Gk[:, 11:16].copy())
    object.__setattr__(out, "XKv43", Gk[:, 16:26].copy())
    object.__setattr__(out, "XKv14", Gk[:, 26:36].copy())
    return out


def _globals_struct(obj) -> GwGlobals:
    g = GwGlobals()
    for n in _lib.GLOBAL_SCALARS:
        setattr(g, n, float(getattr(obj, n)))
    for i in range(5):
        g.Kr[i] = obj.XKr[i]
    for i in range(10):
        g.Kv14[i] = obj.XKv14[i]
        g.Kv43[i] = obj.XKv43[i]
    return g


def _params_struct(obj) -> GwParams:
    p = GwParams()
    for n in _lib.PARAM_NAMES:
        setattr(p, n, getattr(obj, n))
    return p
