"""Ensemble API over the C ABI: many cells of possibly different CRU counts, parameters and
stimulus protocols stepped together on one GB300.

Arrays use the reference's layouts (src/pyGW.cpp:78-87): CaSS [n,4] float64, CaJSR [n] float64,
LCC / LCC_inactivation / ClCh [n,4] int32, RyR [n,4,6] int32.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Dict, Optional, Sequence

import numpy as np

from . import _lib
from ._lib import GwEnsembleDesc, GwGlobals, GwParams, GwStats, GwTrace, check

GLOBAL_NAMES = list(_lib.GLOBAL_SCALARS) + [f"Kr{i}" for i in range(5)] + \
    [f"Kv43_{i}" for i in range(10)] + [f"Kv14_{i}" for i in range(10)]


def _dp(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_int32))


def params_from(obj=None, **overrides) -> GwParams:
    """gw_params from defaults, a GwParams, or any object/dict with the reference's field names."""
    p = _lib.default_params()
    if obj is not None:
        for n in _lib.PARAM_NAMES:
            if isinstance(obj, dict):
                if n in obj:
                    setattr(p, n, obj[n])
            elif hasattr(obj, n):
                setattr(p, n, getattr(obj, n))
    for k, v in overrides.items():
        if k not in _lib.PARAM_NAMES:
            raise ValueError(f"{k} is not a model parameter")
        setattr(p, k, v)
    return p


def globals_to_array(g: GwGlobals) -> np.ndarray:
    return np.frombuffer(bytes(g), dtype=np.float64).copy()


def globals_from_array(a) -> GwGlobals:
    a = np.ascontiguousarray(a, dtype=np.float64)
    if a.size != 36:
        raise ValueError("globals need 36 values")
    return GwGlobals.from_buffer_copy(a.tobytes())


@dataclass
class CRUState:
    CaSS: np.ndarray
    CaJSR: np.ndarray
    LCC: np.ndarray
    LCC_inactivation: np.ndarray
    RyR: np.ndarray
    ClCh: np.ndarray
    JLCC: Optional[np.ndarray] = None

    @classmethod
    def empty(cls, n: int) -> "CRUState":
        return cls(np.zeros((n, 4)), np.zeros(n), np.zeros((n, 4), np.int32),
                   np.zeros((n, 4), np.int32), np.zeros((n, 4, 6), np.int32),
                   np.zeros((n, 4), np.int32), np.zeros((n, 4)))


@dataclass
class Trace:
    t: np.ndarray
    globals: np.ndarray               # [n_cells, n_records, 36]
    crus: Optional[Dict[str, np.ndarray]] = None
    cru_sums: Optional[np.ndarray] = None   # [n_cells, n_records, 8], fields _lib.SUM_FIELDS
    codec: Optional[Dict[str, np.ndarray]] = None  # reduced-memory CRU records of cru_cell
    currents: Optional[np.ndarray] = None  # [n_cells, n_records, 20], fields _lib.CURRENT_FIELDS

    def var(self, name: str) -> np.ndarray:
        return self.globals[..., GLOBAL_NAMES.index(name)]

    def sum(self, name: str) -> np.ndarray:
        return self.cru_sums[..., _lib.SUM_FIELDS.index(name)]

    def current(self, name: str) -> np.ndarray:
        return self.currents[..., _lib.CURRENT_FIELDS.index(name)]


class Ensemble:
    """An ensemble of cells on one device (gw_create / gw_run)."""

    def __init__(self, ncru: Sequence[int], params=None, *, precision: str = "fp32", seed: int = 0,
                 device: int = 0, event_cap: int = 0, cluster_ctas=0, cta_crus: int = 0,
                 steps_per_launch: int = 0, ode_fp32_rhs: bool = False, tune_steps: int = 200,
                 cell_base: int = 0):
        """cluster_ctas: CTAs per cluster, 0 for the size rule, or "auto" to measure the fastest
        shape (cluster size and CTA capacity) for these cells first (gw_autotune, tune_steps trial
        steps per candidate).  cell_base: global index of this ensemble's cell 0 in a larger
        ensemble split over contexts (random streams are keyed on the global index)."""
        self.L = _lib.load()
        self.ncru = np.ascontiguousarray(ncru, dtype=np.int32)
        self.n_cells = int(self.ncru.size)
        if precision not in _lib.PRECISION:
            raise ValueError(f"precision must be one of {list(_lib.PRECISION)}")
        self.precision = precision
        if params is None:
            plist = [_lib.default_params()]
        elif isinstance(params, (list, tuple)):
            plist = [p if isinstance(p, GwParams) else params_from(p) for p in params]
            if len(plist) != self.n_cells:
                raise ValueError("need one parameter set per cell")
        else:
            plist = [params if isinstance(params, GwParams) else params_from(params)]
        self._params = (GwParams * len(plist))(*plist)
        d = GwEnsembleDesc()
        d.n_cells = self.n_cells
        d.ncru = self.ncru.ctypes.data_as(C.POINTER(C.c_int32))
        d.params = C.cast(self._params, C.POINTER(GwParams))
        d.params_per_cell = 1 if len(plist) > 1 else 0
        d.precision = _lib.PRECISION[precision]
        d.seed = seed & 0xFFFFFFFFFFFFFFFF
        d.device = device
        d.event_cap = event_cap
        d.cell_base = int(cell_base)
        self.cell_base = int(cell_base)
        self.global_cells = range(self.cell_base, self.cell_base + self.n_cells)
        self.tuned_us_per_step = None
        if cluster_ctas == "auto":
            best, tile, us = C.c_int(), C.c_int(), C.c_double()
            check(self.L.gw_autotune(C.byref(d), int(tune_steps), C.byref(best), C.byref(tile), C.byref(us)))
            cluster_ctas, cta_crus = best.value, tile.value
            self.tuned_us_per_step = us.value
        d.cluster_ctas = int(cluster_ctas)
        d.cta_crus = cta_crus
        d.steps_per_launch = steps_per_launch
        d.ode_fp32_rhs = 1 if ode_fp32_rhs else 0
        h = C.c_void_p()
        check(self.L.gw_create(C.byref(d), C.byref(h)))
        self.h = h

    @staticmethod
    def partition_spec(ncru: Sequence[int], world: int, rank: int, precision: str = "fp32",
                       cluster_ctas: int = 0, cta_crus: int = 0):
        """(begin, end, cluster_ctas, cta_crus) of this rank's contiguous share of an ensemble of
        len(ncru) cells (dist.partition) and the launch shape every share takes: the whole
        ensemble's (gw_default_shape), since a cell's CRU split depends on the shape.  No device."""
        from .dist import partition

        if cluster_ctas == "auto":
            raise ValueError("tune the whole ensemble once (gw_autotune) and pass its cluster_ctas and cta_crus")
        b, e = partition(len(ncru), world, rank)
        n_all = np.ascontiguousarray(ncru, dtype=np.int32)
        d = GwEnsembleDesc()
        d.n_cells = int(n_all.size)
        d.ncru = n_all.ctypes.data_as(C.POINTER(C.c_int32))
        d.precision = _lib.PRECISION[precision]
        d.cluster_ctas = int(cluster_ctas)
        d.cta_crus = int(cta_crus)
        cl, tile = C.c_int(), C.c_int()
        check(_lib.load().gw_default_shape(C.byref(d), C.byref(cl), C.byref(tile)))
        return b, e, cl.value, tile.value

    @classmethod
    def partitioned(cls, ncru: Sequence[int], params=None, *, world: int, rank: int, **kw) -> "Ensemble":
        """This rank's share of an ensemble of len(ncru) cells (partition_spec), keyed on the cells'
        global indices (cell_base): the union over ranks reproduces one context holding every cell,
        bit for bit.  ``params``: one set for all cells or one per cell (the share is taken);
        ``global_cells`` on the result gives the share's global indices."""
        b, e, cl, tile = cls.partition_spec(ncru, world, rank, kw.get("precision", "fp32"),
                                            kw.get("cluster_ctas", 0), kw.get("cta_crus", 0))
        if e <= b:
            raise ValueError(f"rank {rank} of {world} has no cells of {len(ncru)}")
        if isinstance(params, (list, tuple)):
            if len(params) != len(ncru):
                raise ValueError("need one parameter set per cell")
            params = list(params[b:e])
        kw = dict(kw, cluster_ctas=cl, cta_crus=tile)
        return cls(list(ncru)[b:e], params, cell_base=b, **kw)

    def close(self):
        if getattr(self, "h", None):
            self.L.gw_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---- state ----
    def set_globals(self, cell: int, g):
        if not isinstance(g, GwGlobals):
            g = globals_from_array(g)
        check(self.L.gw_set_globals(self.h, cell, C.byref(g)), self.h)

    def get_globals(self, cell: int) -> np.ndarray:
        g = GwGlobals()
        check(self.L.gw_get_globals(self.h, cell, C.byref(g)), self.h)
        return globals_to_array(g)

    def set_crus(self, cell: int, s: CRUState, with_jlcc: bool = False):
        n = int(self.ncru[cell])
        f = lambda a, dt, shape: np.ascontiguousarray(a, dtype=dt).reshape(shape)
        CaSS = f(s.CaSS, np.float64, (n, 4))
        CaJSR = f(s.CaJSR, np.float64, (n,))
        LCC = f(s.LCC, np.int32, (n, 4))
        LCCi = f(s.LCC_inactivation, np.int32, (n, 4))
        RyR = f(s.RyR, np.int32, (n, 4, 6))
        ClCh = f(s.ClCh, np.int32, (n, 4))
        JLCC = f(s.JLCC, np.float64, (n, 4)) if (with_jlcc and s.JLCC is not None) else None
        check(self.L.gw_set_crus(self.h, cell, _dp(CaSS), _dp(CaJSR), _ip(LCC), _ip(LCCi), _ip(RyR),
                                 _ip(ClCh), _dp(JLCC)), self.h)

    def get_crus(self, cell: int) -> CRUState:
        s = CRUState.empty(int(self.ncru[cell]))
        check(self.L.gw_get_crus(self.h, cell, _dp(s.CaSS), _dp(s.CaJSR), _ip(s.LCC),
                                 _ip(s.LCC_inactivation), _ip(s.RyR), _ip(s.ClCh), _dp(s.JLCC)), self.h)
        return s

    def sample_initial_crus(self, cell: int):
        check(self.L.gw_sample_initial_crus(self.h, cell), self.h)

    def set_flux_carry(self, cell: int, sum_jlcc: float, sum_clch: float, sum_jtr: float,
                       sum_jxfer: float):
        check(self.L.gw_set_flux_carry(self.h, cell, sum_jlcc, sum_clch, sum_jtr, sum_jxfer), self.h)

    def get_flux_carry(self, cell: int):
        """(sum JLCC, sum ClCh, sum Jtr, sum Jxfer) that the next global step uses."""
        v = [C.c_double() for _ in range(4)]
        check(self.L.gw_get_flux_carry(self.h, cell, *[C.byref(x) for x in v]), self.h)
        return tuple(x.value for x in v)

    def time(self, cell: int = 0):
        t, s = C.c_double(), C.c_uint64()
        check(self.L.gw_get_time(self.h, cell, C.byref(t), C.byref(s)), self.h)
        return t.value, int(s.value)

    def set_time(self, cell: int, t: float, step: int):
        check(self.L.gw_set_time(self.h, cell, t, int(step)), self.h)

    def checkpoint(self, cell: int) -> dict:
        """Everything needed to resume a cell bit for bit (globals, CRU arrays with JLCC, flux
        carry, time and RNG step)."""
        t, step = self.time(cell)
        return {"globals": self.get_globals(cell), "crus": self.get_crus(cell),
                "carry": self.get_flux_carry(cell), "t": t, "step": step}

    def restore(self, cell: int, ck: dict):
        self.set_globals(cell, ck["globals"])
        self.set_crus(cell, ck["crus"], with_jlcc=True)
        self.set_flux_carry(cell, *ck["carry"])
        self.set_time(cell, ck["t"], ck["step"])

    # ---- stimulus ----
    def set_pulse(self, start: float = 0.0, period: float = 0.0, duration: float = 0.5,
                  amplitude: float = 100.0, cell: int = -1):
        check(self.L.gw_set_stimulus_pulse(self.h, cell, start, period, duration, amplitude), self.h)

    def set_samples(self, istim, cell: int = -1):
        a = np.ascontiguousarray(istim, dtype=np.float64)
        check(self.L.gw_set_stimulus_samples(self.h, cell, _dp(a), a.size), self.h)

    # ---- stepping ----
    def run(self, dt: float, n_steps: int, record_every: int = 0, cru_cell: Optional[int] = None,
            max_records: Optional[int] = None, sums: bool = False, codec: bool = False,
            currents: bool = False) -> Optional[Trace]:
        """Advance every cell by n_steps.  With record_every > 0, returns the globals of every cell
        at each record; cru_cell adds that cell's CRU arrays (codec=True: in the reduced-memory
        layout, written by the device); sums=True adds every cell's record-time CRU sums;
        currents=True the reference's GWSolution currents of every record, evaluated on the device."""
        if record_every <= 0:
            check(self.L.gw_run(self.h, dt, int(n_steps), 0, None), self.h)
            return None
        nrec = n_steps // record_every if max_records is None else max_records
        tr = GwTrace()
        tr.max_records = nrec
        t = np.zeros(max(nrec, 1))
        G = np.zeros((self.n_cells, max(nrec, 1), 36))
        tr.t = _dp(t)
        tr.globals = _dp(G)
        tr.cru_cell = -1
        crus = None
        cod = None
        cs = None
        if sums:
            cs = np.zeros((self.n_cells, max(nrec, 1), _lib.CRU_SUMS))
            tr.cru_sums = _dp(cs)
        cur = None
        if currents:
            cur = np.zeros((self.n_cells, max(nrec, 1), len(_lib.CURRENT_FIELDS)))
            tr.currents = _dp(cur)
        if cru_cell is not None and codec:
            n = int(self.ncru[cru_cell])
            cod = {"LCC": np.zeros((nrec, n, 4), np.int8), "LCC_inactivation": np.zeros((nrec, n, 4), np.bool_),
                   "ClCh": np.zeros((nrec, n, 4), np.bool_), "RyR": np.zeros((nrec, n, 4), np.int16),
                   "CaSS": np.zeros((nrec, n, 4), np.float32), "CaJSR": np.zeros((nrec, n), np.float32)}
            tr.cru_cell = cru_cell
            tr.LCC_i8 = cod["LCC"].ctypes.data_as(C.POINTER(C.c_int8))
            tr.LCC_inactivation_u8 = cod["LCC_inactivation"].ctypes.data_as(C.POINTER(C.c_uint8))
            tr.ClCh_u8 = cod["ClCh"].ctypes.data_as(C.POINTER(C.c_uint8))
            tr.RyR_i16 = cod["RyR"].ctypes.data_as(C.POINTER(C.c_int16))
            tr.CaSS_f32 = cod["CaSS"].ctypes.data_as(C.POINTER(C.c_float))
            tr.CaJSR_f32 = cod["CaJSR"].ctypes.data_as(C.POINTER(C.c_float))
        elif cru_cell is not None:
            n = int(self.ncru[cru_cell])
            crus = {"CaSS": np.zeros((nrec, n, 4)), "CaJSR": np.zeros((nrec, n)),
                    "LCC": np.zeros((nrec, n, 4), np.int32),
                    "LCC_inactivation": np.zeros((nrec, n, 4), np.int32),
                    "RyR": np.zeros((nrec, n, 4, 6), np.int32), "ClCh": np.zeros((nrec, n, 4), np.int32)}
            tr.cru_cell = cru_cell
            tr.CaSS, tr.CaJSR = _dp(crus["CaSS"]), _dp(crus["CaJSR"])
            tr.LCC, tr.LCC_inactivation = _ip(crus["LCC"]), _ip(crus["LCC_inactivation"])
            tr.RyR, tr.ClCh = _ip(crus["RyR"]), _ip(crus["ClCh"])
        check(self.L.gw_run(self.h, dt, int(n_steps), record_every, C.byref(tr)), self.h)
        k = int(tr.n_written)
        if crus is not None:
            crus = {a: b[:k] for a, b in crus.items()}
        if cod is not None:
            cod = {a: b[:k] for a, b in cod.items()}
        return Trace(t=t[:k], globals=G[:, :k], crus=crus, cru_sums=None if cs is None else cs[:, :k], codec=cod,
                     currents=None if cur is None else cur[:, :k])

    def stats(self) -> dict:
        s = GwStats()
        check(self.L.gw_get_stats(self.h, C.byref(s)), self.h)
        return {f: getattr(s, f) for f, _ in GwStats._fields_}
