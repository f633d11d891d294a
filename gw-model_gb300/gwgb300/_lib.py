"""ctypes bindings of the engine's C ABI (include/gw_gb300.h).

The library is the in-tree ``gw-model_gb300/_build/libgwgb300.so``; there is no fallback: if it
is missing or no sm_103 device is present, calls raise.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import _build

# GW::Parameters (GW_utils.hpp:38-160): member order of gw_params.
PARAM_NAMES = (
    "T CSA Vcyto VNSR VJSR VSS NCaRU Ko Nao Cao Clo Clcyto f g f1 g1 a b gamma0 omega PCaL kfClCh "
    "kbClCh Pto2 k12 k21 k23 k32 k34 k43 k45 k54 k56 k65 k25 k52 rRyR rxfer rtr riss BSRT KBSR "
    "BSLT KBSL CSQNT KCSQN CMDNT KCMDN GNa GKr Kf Kb GKs GKv43 alphaa0Kv43 aaKv43 betaa0Kv43 "
    "baKv43 alphai0Kv43 aiKv43 betai0Kv43 biKv43 f1Kv43 f2Kv43 f3Kv43 f4Kv43 b1Kv43 b2Kv43 "
    "b3Kv43 b4Kv43 PKv14 alphaa0Kv14 aaKv14 betaa0Kv14 baKv14 alphai0Kv14 aiKv14 betai0Kv14 "
    "biKv14 f1Kv14 f2Kv14 f3Kv14 f4Kv14 b1Kv14 b2Kv14 b3Kv14 b4Kv14 Csc GK1 KmK1 GKp kNaCa KmNa "
    "KmCa ksat eta INaKmax KmNai KmKo IpCamax KmpCa GCab GNab kHTRPNp kHTRPNm kLTRPNp kLTRPNm "
    "HTRPNtot LTRPNtot Vmaxf Vmaxr Kmf Kmr Hf Hr").split()

GLOBAL_SCALARS = ("V", "Nai", "Ki", "Cai", "CaNSR", "CaLTRPN", "CaHTRPN", "m", "h", "j", "xKs")

GW_OK = 0
GW_ERR_INVALID_ARGUMENT = 1
GW_ERR_CUDA = 2
GW_ERR_NO_DEVICE = 3
GW_ERR_EVENT_CAP = 4
GW_ERR_NONFINITE = 5
GW_ERR_NERNST = 6
GW_ERR_UNSUPPORTED = 7
GW_ERR_OUT_OF_MEMORY = 8
GW_ERR_SYNC_TIMEOUT = 9

PRECISION = {"fp64": 0, "fp32": 1}


class GwParams(C.Structure):
    _fields_ = [(n, C.c_int if n == "NCaRU" else C.c_double) for n in PARAM_NAMES]


class GwGlobals(C.Structure):
    _fields_ = [(n, C.c_double) for n in GLOBAL_SCALARS] + [
        ("Kr", C.c_double * 5), ("Kv43", C.c_double * 10), ("Kv14", C.c_double * 10)]


class GwEnsembleDesc(C.Structure):
    _fields_ = [("n_cells", C.c_int), ("ncru", C.POINTER(C.c_int32)), ("params", C.POINTER(GwParams)),
                ("params_per_cell", C.c_int), ("precision", C.c_int), ("seed", C.c_uint64),
                ("device", C.c_int), ("event_cap", C.c_int), ("cluster_ctas", C.c_int),
                ("cta_crus", C.c_int), ("steps_per_launch", C.c_int), ("ode_fp32_rhs", C.c_int),
                ("cell_base", C.c_int)]


class GwTrace(C.Structure):
    _fields_ = [("max_records", C.c_int64), ("t", C.POINTER(C.c_double)),
                ("globals", C.POINTER(C.c_double)), ("cru_cell", C.c_int),
                ("CaSS", C.POINTER(C.c_double)), ("CaJSR", C.POINTER(C.c_double)),
                ("LCC", C.POINTER(C.c_int32)), ("LCC_inactivation", C.POINTER(C.c_int32)),
                ("RyR", C.POINTER(C.c_int32)), ("ClCh", C.POINTER(C.c_int32)),
                ("n_written", C.c_int64), ("cru_sums", C.POINTER(C.c_double)),
                ("LCC_i8", C.POINTER(C.c_int8)), ("LCC_inactivation_u8", C.POINTER(C.c_uint8)),
                ("ClCh_u8", C.POINTER(C.c_uint8)), ("RyR_i16", C.POINTER(C.c_int16)),
                ("CaSS_f32", C.POINTER(C.c_float)), ("CaJSR_f32", C.POINTER(C.c_float)),
                ("currents", C.POINTER(C.c_double))]


CRU_SUMS = 8
# Last axis of gw_trace.currents (GW_CUR_* order): the reference's GWSolution currents, evaluated on the device.
CURRENT_FIELDS = ["INa", "INab", "IKr", "IKs", "IKv43", "IKv14", "Ito1", "IK1", "IKp", "INaK", "INaCa", "IpCa",
                  "ICab", "Jup", "ICaL", "Ito2", "Jtr", "Jxfer", "LCC_open_fraction", "RyR_open_fraction"]
SUM_FIELDS = ["LCC_open", "LCC_conducting", "CaSS_conducting", "RyR_open", "ClCh_open", "CaSS", "CaJSR", "CRUs"]


class GwStats(C.Structure):
    _fields_ = [("steps", C.c_uint64), ("launches", C.c_uint64), ("kernel_ms", C.c_double),
                ("events", C.c_uint64), ("cluster_ctas", C.c_int), ("cta_crus", C.c_int),
                ("threads_per_cta", C.c_int), ("n_clusters", C.c_int), ("ctas", C.c_int),
                ("device_allocs", C.c_uint64)]


# Parameters of the gradient path (GW_TH_* order) and the gw_params fields each one scales.
GRAD_THETA = ("PCaL", "GKr", "GKs", "GK1", "INaKmax", "Vmax", "rRyR", "CSQNT")
GRAD_THETA_FIELDS = (("PCaL",), ("GKr",), ("GKs",), ("GK1",), ("INaKmax",), ("Vmaxf", "Vmaxr"), ("rRyR",),
                     ("CSQNT",))


class GwGradDesc(C.Structure):
    _fields_ = [("n_cells", C.c_int), ("ncru", C.POINTER(C.c_int32)), ("params", C.POINTER(GwParams)),
                ("params_per_cell", C.c_int), ("seed", C.c_uint64), ("device", C.c_int), ("dt", C.c_double),
                ("n_steps", C.c_int64), ("checkpoint_every", C.c_int), ("sample_every", C.c_int),
                ("stim", C.POINTER(C.c_double)), ("event_cap", C.c_int), ("cell_base", C.c_int)]


class GwGradStats(C.Structure):
    _fields_ = [("forward_ms", C.c_double), ("backward_ms", C.c_double), ("replay_ms", C.c_double),
                ("events", C.c_int64), ("checkpoint_bytes", C.c_int64), ("segment_bytes", C.c_int64)]


# Exported entry points and their signatures (all return int status unless noted).
_P = C.POINTER
_SIGS = {
    "gw_abi_version": ([], C.c_int),
    "gw_params_default": ([_P(GwParams)], None),
    "gw_globals_default": ([_P(GwGlobals)], None),
    "gw_globals_py_default": ([_P(GwGlobals)], None),
    "gw_create": ([_P(GwEnsembleDesc), _P(C.c_void_p)], C.c_int),
    "gw_destroy": ([C.c_void_p], C.c_int),
    "gw_set_globals": ([C.c_void_p, C.c_int, _P(GwGlobals)], C.c_int),
    "gw_get_globals": ([C.c_void_p, C.c_int, _P(GwGlobals)], C.c_int),
    "gw_set_crus": ([C.c_void_p, C.c_int, _P(C.c_double), _P(C.c_double), _P(C.c_int32),
                     _P(C.c_int32), _P(C.c_int32), _P(C.c_int32), _P(C.c_double)], C.c_int),
    "gw_get_crus": ([C.c_void_p, C.c_int, _P(C.c_double), _P(C.c_double), _P(C.c_int32),
                     _P(C.c_int32), _P(C.c_int32), _P(C.c_int32), _P(C.c_double)], C.c_int),
    "gw_set_flux_carry": ([C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double], C.c_int),
    "gw_get_flux_carry": ([C.c_void_p, C.c_int] + [_P(C.c_double)] * 4, C.c_int),
    "gw_sample_initial_crus": ([C.c_void_p, C.c_int], C.c_int),
    "gw_set_stimulus_pulse": ([C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double], C.c_int),
    "gw_set_stimulus_samples": ([C.c_void_p, C.c_int, _P(C.c_double), C.c_int64], C.c_int),
    "gw_run": ([C.c_void_p, C.c_double, C.c_int64, C.c_int, _P(GwTrace)], C.c_int),
    "gw_run_noalloc": ([C.c_void_p, C.c_double, C.c_int64, C.c_int, _P(GwTrace)], C.c_int),
    "gw_autotune": ([_P(GwEnsembleDesc), C.c_int, _P(C.c_int), _P(C.c_int), _P(C.c_double)], C.c_int),
    "gw_default_shape": ([_P(GwEnsembleDesc), _P(C.c_int), _P(C.c_int)], C.c_int),
    "gw_math_check": ([_P(C.c_double), C.c_int64, _P(C.c_double), _P(C.c_double)], C.c_int),
    "gw_screen_check": ([_P(GwParams), C.c_int, C.c_int64, _P(C.c_uint32), _P(C.c_double), _P(C.c_double),
                         _P(C.c_double), _P(C.c_double), C.c_uint64, _P(C.c_int32), _P(C.c_double)], C.c_int),
    "gw_get_time": ([C.c_void_p, C.c_int, _P(C.c_double), _P(C.c_uint64)], C.c_int),
    "gw_set_time": ([C.c_void_p, C.c_int, C.c_double, C.c_uint64], C.c_int),
    "gw_get_stats": ([C.c_void_p, _P(GwStats)], C.c_int),
    "gw_last_error": ([C.c_void_p, C.c_char_p, C.c_size_t], C.c_int),
    "gw_global_step_host": ([_P(GwParams), C.c_int, _P(C.c_double), _P(C.c_double), C.c_double, C.c_double,
                             _P(C.c_double)], C.c_int),
    "gw_simulate": ([_P(GwParams), C.c_int, C.c_double, C.c_int64, _P(C.c_double), C.c_int,
                     _P(C.c_double), _P(C.c_double), _P(C.c_int32), _P(C.c_int32), _P(C.c_int32),
                     _P(C.c_int32), _P(GwGlobals), C.c_char_p, C.c_uint64, C.c_int, _P(GwTrace)],
                    C.c_int),
    "gw_grad_create": ([_P(GwGradDesc), _P(C.c_void_p)], C.c_int),
    "gw_grad_destroy": ([C.c_void_p], C.c_int),
    "gw_grad_set_state": ([C.c_void_p, C.c_int, _P(GwGlobals), _P(C.c_double), _P(C.c_double), _P(C.c_int32),
                           _P(C.c_int32), _P(C.c_int32), _P(C.c_int32)], C.c_int),
    "gw_grad_forward": ([C.c_void_p, _P(C.c_double)], C.c_int),
    "gw_grad_backward": ([C.c_void_p, _P(C.c_double), _P(C.c_double)], C.c_int),
    "gw_grad_replay": ([C.c_void_p, C.c_int, _P(C.c_int32), _P(GwParams), _P(C.c_double), _P(C.c_int64)],
                       C.c_int),
    "gw_grad_regime_steps": ([C.c_void_p, _P(C.c_int64)], C.c_int),
    "gw_grad_get_globals": ([C.c_void_p, C.c_int, _P(GwGlobals)], C.c_int),
    "gw_grad_get_stats": ([C.c_void_p, _P(GwGradStats)], C.c_int),
    "gw_grad_last_error": ([C.c_void_p, C.c_char_p, C.c_size_t], C.c_int),
    "gw_grad_check_global": ([_P(GwParams), C.c_int, _P(C.c_double), _P(C.c_double), C.c_double, C.c_double,
                              _P(C.c_double), _P(C.c_double), _P(C.c_double), _P(C.c_double), _P(C.c_double)],
                             C.c_int),
    "gw_grad_check_cru": ([_P(GwParams), C.c_int, _P(C.c_double), _P(C.c_int32), _P(C.c_double), C.c_int,
                           _P(C.c_double), _P(C.c_int32), _P(C.c_int32), _P(C.c_int32), _P(C.c_double),
                           _P(C.c_double), _P(C.c_double), _P(C.c_double), _P(C.c_double), _P(C.c_double),
                           _P(C.c_double)], C.c_int),
}

_lock = threading.Lock()
_lib = None


def lib_path() -> str:
    return _build.LIB_PATH


def load(build_if_missing: bool = True) -> C.CDLL:
    """Load the CUDA library (building it with nvcc if it is missing or stale)."""
    global _lib
    with _lock:
        if _lib is None:
            if build_if_missing:
                _build.build()
            if not os.path.exists(_build.LIB_PATH):
                raise RuntimeError(f"engine library {_build.LIB_PATH} is missing; run the build")
            L = C.CDLL(_build.LIB_PATH)
            for name, (args, res) in _SIGS.items():
                f = getattr(L, name)
                f.argtypes = args
                f.restype = res
            _lib = L
    return _lib


def last_error(ctx=None) -> str:
    buf = C.create_string_buffer(1024)
    load().gw_last_error(ctx, buf, len(buf))
    return buf.value.decode(errors="replace")


class GWError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[gw status {code}] {msg}")
        self.code = code


def check(rc: int, ctx=None) -> None:
    """Map a gw_status to a Python exception (invalid argument -> ValueError)."""
    if rc == GW_OK:
        return
    msg = last_error(ctx)
    if rc == GW_ERR_INVALID_ARGUMENT:
        raise ValueError(msg)
    raise GWError(rc, msg)


def default_params() -> GwParams:
    p = GwParams()
    load().gw_params_default(C.byref(p))
    return p


def default_globals(py: bool = False) -> GwGlobals:
    g = GwGlobals()
    (load().gw_globals_py_default if py else load().gw_globals_default)(C.byref(g))
    return g
