"""GB300 engine for the Greenstein-Winslow (2002) stochastic ventricular myocyte model.

- ``gwgb300.engine.Ensemble``: many cells stepped together on one device (C ABI: gw_create/gw_run).
- ``GreensteinWinslow`` (sibling module): drop-in for the reference's pybind11 module.
"""
from . import _build, _lib  # noqa: F401
from .engine import CRUState, Ensemble, Trace, params_from  # noqa: F401

__all__ = ["Ensemble", "CRUState", "Trace", "params_from"]
