"""Pathwise gradients of a voltage-trace loss over the C ABI (gw_grad_*), and a
``torch.autograd.Function`` over them.

The reference has no derivatives; this is the differentiation path of parameter fits of the model.
An ensemble of cells runs forward on the GB300 with the engine's FP64 SSA lane and draws (the jump
trajectory gw_run would draw), V is sampled every ``sample_every`` steps, and the backward pass
returns for every cell the relative sensitivities theta_k dL/dtheta_k of the 8 parameters of
``THETA`` (PCaL, GKr, GKs, GK1, INaKmax, Vmaxf and Vmaxr together, rRyR, CSQNT).

The estimator is pathwise and conditional on the forward pass's jump trajectory: jump times,
chosen transitions and RyR re-splits are held fixed and only the continuous CRU and global updates
are differentiated.  It ignores how the jump times and transition choices depend on the
parameters, so it is the derivative of the frozen-trajectory replay (``GradEngine.replay``), not of
the expected loss.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import List, Sequence, Tuple

import numpy as np
import torch

from . import _lib
from ._lib import GwGlobals, GwGradDesc, GwGradStats, GwParams
from .engine import CRUState, Ensemble, globals_from_array, params_from

THETA = _lib.GRAD_THETA


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


def scaled_params(base: GwParams, scales) -> GwParams:
    """A copy of ``base`` with each parameter of THETA multiplied by its scale."""
    s = np.asarray(scales, dtype=np.float64)
    if s.shape != (len(THETA),):
        raise ValueError(f"need {len(THETA)} scales")
    p = GwParams.from_buffer_copy(bytes(base))
    for k, names in enumerate(_lib.GRAD_THETA_FIELDS):
        for n in names:
            setattr(p, n, getattr(base, n) * float(s[k]))
    return p


def initial_states(ncru: Sequence[int], seed: int, params=None, device: int = 0) -> List[CRUState]:
    """The reference's random initial CRU state (GW_utils.tpp:5-64) of each cell, drawn on the device
    from the engine's stream for (seed, cell)."""
    with Ensemble(ncru, params, precision="fp64", seed=seed, device=device) as e:
        out = []
        for c in range(e.n_cells):
            e.sample_initial_crus(c)
            out.append(e.get_crus(c))
    return out


def _check(L, rc: int, h) -> None:
    if rc == _lib.GW_OK:
        return
    buf = C.create_string_buffer(1024)
    L.gw_grad_last_error(h, buf, len(buf))
    msg = buf.value.decode(errors="replace")
    if rc == _lib.GW_ERR_INVALID_ARGUMENT:
        raise ValueError(msg)
    raise _lib.GWError(rc, msg)


class GradEngine:
    """Forward pass, adjoint and frozen-trajectory replay of an ensemble of cells (gw_grad_*)."""

    def __init__(self, ncru: Sequence[int], params=None, *, n_steps: int, dt: float = 1e-3, seed: int = 0,
                 checkpoint_every: int = 200, sample_every: int = 500,
                 stim: Sequence[float] | np.ndarray = (0.0, 0.0, 0.5, 100.0), device: int = 0,
                 event_cap: int = 0, cell_base: int = 0):
        """params: one GwParams (or mapping) for all cells, or a list with one per cell.  stim: the
        pulse train (start, period, duration, amplitude) of every cell, or one row per cell."""
        self.L = _lib.load()
        self.h = None
        self.ncru = np.ascontiguousarray(ncru, dtype=np.int32)
        self.n_cells = int(self.ncru.size)
        if isinstance(params, (list, tuple)):
            plist = [p if isinstance(p, GwParams) else params_from(p) for p in params]
            if len(plist) != self.n_cells:
                raise ValueError("need one parameter set per cell")
        else:
            plist = [params if isinstance(params, GwParams) else params_from(params)]
        self.params = plist
        self._params = (GwParams * len(plist))(*plist)
        st = np.asarray(stim, dtype=np.float64)
        if st.ndim == 1:
            st = np.tile(st, (self.n_cells, 1))
        if st.shape != (self.n_cells, 4):
            raise ValueError("stim needs (start, period, duration, amplitude) per cell")
        self.stim = np.ascontiguousarray(st)
        self.n_steps = int(n_steps)
        self.sample_every = int(sample_every)
        self.n_samples = self.n_steps // self.sample_every
        d = GwGradDesc()
        d.n_cells = self.n_cells
        d.ncru = _ip(self.ncru)
        d.params = C.cast(self._params, C.POINTER(GwParams))
        d.params_per_cell = 1 if len(plist) > 1 else 0
        d.seed = seed & 0xFFFFFFFFFFFFFFFF
        d.device = device
        d.dt = dt
        d.n_steps = self.n_steps
        d.checkpoint_every = checkpoint_every
        d.sample_every = self.sample_every
        d.stim = _dp(self.stim)
        d.event_cap = event_cap
        d.cell_base = int(cell_base)
        h = C.c_void_p()
        _check(self.L, self.L.gw_grad_create(C.byref(d), C.byref(h)), None)
        self.h = h

    def close(self):
        if self.h is not None:
            self.L.gw_grad_destroy(self.h)
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

    def set_state(self, cell: int, globals_, crus: CRUState):
        g = globals_ if isinstance(globals_, GwGlobals) else globals_from_array(globals_)
        a = {k: np.ascontiguousarray(getattr(crus, k), np.float64 if k in ("CaSS", "CaJSR") else np.int32)
             for k in ("CaSS", "CaJSR", "LCC", "LCC_inactivation", "RyR", "ClCh")}
        n = int(self.ncru[cell])
        if a["CaSS"].shape != (n, 4) or a["RyR"].shape != (n, 4, 6):
            raise ValueError(f"cell {cell} has {n} CRUs")
        _check(self.L, self.L.gw_grad_set_state(self.h, cell, C.byref(g), _dp(a["CaSS"]), _dp(a["CaJSR"]),
                                                _ip(a["LCC"]), _ip(a["LCC_inactivation"]), _ip(a["RyR"]),
                                                _ip(a["ClCh"])), self.h)

    def forward(self) -> np.ndarray:
        """V [n_cells, n_samples] after steps sample_every - 1, 2 sample_every - 1, ..."""
        V = np.zeros((self.n_cells, max(1, self.n_samples)))
        _check(self.L, self.L.gw_grad_forward(self.h, _dp(V)), self.h)
        return V[:, :self.n_samples]

    def backward(self, dL_dV) -> np.ndarray:
        """dL/dV [n_cells, n_samples] -> relative sensitivities [n_cells, 8] (THETA order)."""
        g = np.ascontiguousarray(dL_dV, dtype=np.float64)
        if g.shape != (self.n_cells, self.n_samples):
            raise ValueError(f"dL_dV must be {(self.n_cells, self.n_samples)}")
        sens = np.zeros((self.n_cells, len(THETA)))
        _check(self.L, self.L.gw_grad_backward(self.h, _dp(g), _dp(sens)), self.h)
        return sens

    def replay(self, src: Sequence[int], params: Sequence, regime: bool = False):
        """Frozen-trajectory replay: variant v re-runs cell src[v] with params[v] on that cell's jump
        trajectory.  Returns V [n_var, n_samples] (and, with regime, the steps each variant began
        at V >= -40 mV)."""
        s = np.ascontiguousarray(src, dtype=np.int32)
        plist = [p if isinstance(p, GwParams) else params_from(p) for p in params]
        if len(plist) != s.size:
            raise ValueError("need one parameter set per variant")
        P = (GwParams * len(plist))(*plist)
        V = np.zeros((s.size, max(1, self.n_samples)))
        R = np.zeros(s.size, np.int64)
        _check(self.L, self.L.gw_grad_replay(self.h, int(s.size), _ip(s), C.cast(P, C.POINTER(GwParams)), _dp(V),
                                             R.ctypes.data_as(C.POINTER(C.c_int64))), self.h)
        V = V[:, :self.n_samples]
        return (V, R) if regime else V

    def regime_steps(self) -> np.ndarray:
        R = np.zeros(self.n_cells, np.int64)
        _check(self.L, self.L.gw_grad_regime_steps(self.h, R.ctypes.data_as(C.POINTER(C.c_int64))), self.h)
        return R

    def final_globals(self, cell: int) -> np.ndarray:
        g = GwGlobals()
        _check(self.L, self.L.gw_grad_get_globals(self.h, cell, C.byref(g)), self.h)
        return np.frombuffer(bytes(g), dtype=np.float64).copy()

    def stats(self) -> dict:
        s = GwGradStats()
        _check(self.L, self.L.gw_grad_get_stats(self.h, C.byref(s)), self.h)
        return {k: getattr(s, k) for k, _ in GwGradStats._fields_}


@dataclass
class TraceSpec:
    """A voltage-trace experiment for VoltageTrace: cells, base parameters, initial states and
    protocol.  ``states`` holds (globals, CRUState) per cell."""
    ncru: Sequence[int]
    base: GwParams
    states: List[Tuple[object, CRUState]]
    seed: int
    n_steps: int
    dt: float = 1e-3
    checkpoint_every: int = 200
    sample_every: int = 500
    stim: Sequence[float] = (0.0, 0.0, 0.5, 100.0)
    device: int = 0
    engines: list = field(default_factory=list, repr=False)

    def build(self, scales: np.ndarray) -> GradEngine:
        """A GradEngine whose cell c has the base parameters scaled by scales[c] (THETA order)."""
        scales = np.asarray(scales, dtype=np.float64).reshape(len(self.ncru), len(THETA))
        plist = [scaled_params(self.base, scales[c]) for c in range(len(self.ncru))]
        e = GradEngine(self.ncru, plist, n_steps=self.n_steps, dt=self.dt, seed=self.seed,
                       checkpoint_every=self.checkpoint_every, sample_every=self.sample_every,
                       stim=self.stim, device=self.device)
        for c, (g, s) in enumerate(self.states):
            e.set_state(c, g, s)
        return e


class VoltageTrace(torch.autograd.Function):
    """V samples [n_cells, n_samples] of a TraceSpec as a function of per-cell parameter scales
    [n_cells, 8] (float64).  Backward: dL/dscale_k = (theta_k dL/dtheta_k) / scale_k, pathwise and
    conditional on the forward pass's jump trajectory."""

    @staticmethod
    def forward(ctx, scales: torch.Tensor, spec: TraceSpec):
        eng = spec.build(scales.detach().cpu().numpy())
        V = eng.forward()
        ctx.eng = eng
        ctx.save_for_backward(scales)
        return torch.from_numpy(V).to(device=scales.device, dtype=torch.float64)

    @staticmethod
    def backward(ctx, gV: torch.Tensor):
        (scales,) = ctx.saved_tensors
        eng = ctx.eng
        sens = eng.backward(gV.detach().to("cpu", torch.float64).numpy())
        eng.close()
        ctx.eng = None
        return torch.from_numpy(sens).to(scales) / scales, None
