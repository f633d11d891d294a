"""ctypes bindings for the CPU oracle (TEST INFRASTRUCTURE ONLY).

Loads ``oracle/_build/liboracle.so`` (the C restatement of the reference's hot path, gw_oracle.c)
and, when it has been built in a container that holds the reference sources,
``oracle/_ref/libgwref.so`` (the reference's own C++ with injected draws).  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg import this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
# the same C source built with the reference's Release flags (CPU baseline timings only)
TIMED_LIB_PATH = os.path.join(HERE, "_build", "liboracle_timed.so")
REF_PATH = os.path.join(HERE, "_ref", "libgwref.so")
REF_TIMED_PATH = os.path.join(HERE, "_ref", "libgwref_timed.so")

U53, U24 = 0, 1

# (type, name, default): the reference's Parameters struct, GW_utils.hpp:40-156.
_PARAM_TABLE = None


def _parse_param_table():
    global _PARAM_TABLE
    if _PARAM_TABLE is None:
        import re

        src = open(os.path.join(HERE, "gw_oracle.h")).read()
        body = src[src.index("#define ORC_PARAM_FIELDS(X)"):src.index("#define ORC_DECL_FIELD")]
        _PARAM_TABLE = [(t, n, float(d)) for t, n, d in
                        re.findall(r"X\((double|int),\s*(\w+),\s*([-+0-9.eE]+)\)", body)]
    return _PARAM_TABLE


def param_table():
    return list(_parse_param_table())


class OrcParams(C.Structure):
    _fields_ = [(n, C.c_int if t == "int" else C.c_double) for t, n, _ in _parse_param_table()]


GLOBAL_SCALARS = ["V", "Nai", "Ki", "Cai", "CaNSR", "CaLTRPN", "CaHTRPN", "m", "h", "j", "xKs"]


class OrcGlobals(C.Structure):
    _fields_ = [(n, C.c_double) for n in GLOBAL_SCALARS] + [
        ("Kr", C.c_double * 5), ("Kv43", C.c_double * 10), ("Kv14", C.c_double * 10)]

    def to_array(self) -> np.ndarray:
        return np.frombuffer(bytes(self), dtype=np.float64).copy()

    @classmethod
    def from_array(cls, a) -> "OrcGlobals":
        a = np.ascontiguousarray(a, dtype=np.float64)
        assert a.size == 36
        return cls.from_buffer_copy(a.tobytes())


CONST_NAMES = ("RT_F F_RT CRU_factor CSA_FVcyto VSS_Vcyto Vcyto_VNSR VJSR_VNSR a gamma0 gamma0a "
               "gamma0a2 gamma0a3 gamma0a4 binv omega omega_b omega_b2 omega_b3 omega_b4 BSR_const "
               "BSL_const VSS_VJSR CSQN_const JLCC_const Cao_scaled Nao3 INaCa_const sigma "
               "INaK_const sqrtKo PKv14_Csc Ito2_const IK1_const ICaL_const CMDN_const VF_RT "
               "expmVF_RT ENa EK ECa beta_cyto JLCC_multiplier JLCC_exp alphaLCC betaLCC yinfLCC "
               "tauLCC").split()
CURRENT_NAMES = ("INa INab INaCa INaK IKr IKs Ito1 Ito2 IK1 IKp ICaL ICab IpCa Jup Jtr_tot "
                 "Jxfer_tot").split()


class OrcConsts(C.Structure):
    _fields_ = [(n, C.c_double) for n in CONST_NAMES]


class OrcCurrents(C.Structure):
    _fields_ = [(n, C.c_double) for n in CURRENT_NAMES]


_lock = threading.Lock()
_lib = None
_timed = None
_ref = None


def reference_dir() -> str:
    """Checkout of the reference (lukeoloughlin/GW-model): $GW_REFERENCE_DIR, else the REF default
    of oracle/Makefile, the recipe that compiles the reference's sources where they lie."""
    env = os.environ.get("GW_REFERENCE_DIR")
    if env:
        return env
    import re

    with open(os.path.join(HERE, "Makefile")) as f:
        m = re.search(r"^REF\s*\?=\s*(\S+)", f.read(), re.M)
    return m.group(1) if m else ""


def reference_sources_present() -> bool:
    return os.path.isdir(os.path.join(reference_dir(), "src", "includes"))


def build(force: bool = False) -> None:
    """Compile the oracle (and the reference harness when the reference sources are present)."""
    with _lock:
        if force or not os.path.exists(LIB_PATH):
            subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
        if reference_sources_present() and (force or not os.path.exists(REF_PATH)):
            subprocess.run(["make", "-s", "-C", HERE, "ref", "REF=" + reference_dir()], check=True)


def _dp(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_int))


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = _bind(C.CDLL(LIB_PATH))
    return _lib


def timed_lib():
    """gw_oracle.c built with the reference's Release flags (-Ofast -funroll-loops): the CPU
    baseline's timings use it; its results are not bit-exact with the parity build."""
    global _timed
    if _timed is None:
        if not os.path.exists(TIMED_LIB_PATH):
            build(force=True)
        _timed = _bind(C.CDLL(TIMED_LIB_PATH))
    return _timed


def _bind(L):
    if True:
        vp = C.c_void_p
        P = C.POINTER
        L.orc_params_default.argtypes = [P(OrcParams)]
        L.orc_globals_default.argtypes = [P(OrcGlobals)]
        L.orc_globals_py_default.argtypes = [P(OrcGlobals)]
        L.orc_constants.argtypes = [P(OrcParams), C.c_int, P(OrcConsts)]
        L.orc_philox4x32_10.argtypes = [P(C.c_uint32), P(C.c_uint32), P(C.c_uint32)]
        L.orc_uniforms.argtypes = [C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint64, C.c_uint32,
                                   C.c_int, C.c_uint32, C.c_int, P(C.c_double)]
        L.orc_cru_rates.argtypes = [P(OrcParams), P(OrcConsts)] + [P(C.c_int)] * 4 + [P(C.c_double)] * 6
        L.orc_ssa_step_constants.argtypes = [P(OrcConsts), C.c_double]
        L.orc_create.restype = vp
        L.orc_create.argtypes = [P(OrcParams), C.c_int, C.c_uint64, C.c_uint32, C.c_int]
        L.orc_destroy.argtypes = [vp]
        L.orc_set_globals.argtypes = [vp, P(OrcGlobals)]
        L.orc_get_globals.argtypes = [vp, P(OrcGlobals)]
        L.orc_set_crus.argtypes = [vp, P(C.c_double), P(C.c_double)] + [P(C.c_int)] * 4
        L.orc_get_crus.argtypes = [vp, P(C.c_double), P(C.c_double)] + [P(C.c_int)] * 4
        L.orc_set_fluxes.argtypes = [vp] + [P(C.c_double)] * 3
        L.orc_get_fluxes.argtypes = [vp] + [P(C.c_double)] * 3
        L.orc_get_consts.argtypes = [vp, P(OrcConsts)]
        L.orc_get_currents.argtypes = [vp, P(OrcCurrents)]
        L.orc_set_step.argtypes = [vp, C.c_uint64]
        L.orc_get_step.restype = C.c_uint64
        L.orc_get_step.argtypes = [vp]
        L.orc_sample_initial_crus.argtypes = [vp]
        L.orc_euler_step.argtypes = [vp, C.c_double, C.c_double]
        L.orc_run.restype = C.c_int64
        L.orc_run.argtypes = [vp, C.c_double, C.c_int64, P(C.c_double), C.c_int, C.c_int64,
                              P(C.c_double), P(OrcGlobals)]
        L.orc_run_record.restype = C.c_int64
        L.orc_run_record.argtypes = [vp, C.c_double, C.c_int64, P(C.c_double), C.c_int, C.c_int64,
                                     P(C.c_double), P(OrcGlobals), P(C.c_double), P(C.c_double)] + \
            [P(C.c_int)] * 4
        L.orc_event_count.restype = C.c_int64
        L.orc_event_count.argtypes = [vp]
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_param_count.restype = C.c_int
    return L


def ref_available() -> bool:
    return os.path.exists(REF_PATH)


def ref_lib():
    """The reference's own C++ with injected draws (exists only where the reference was built)."""
    global _ref
    if _ref is None:
        L = C.CDLL(REF_PATH)
        vp = C.c_void_p
        P = C.POINTER
        L.ref_create.restype = vp
        L.ref_create.argtypes = [P(OrcParams), C.c_int, C.c_uint64, C.c_uint32, C.c_int]
        L.ref_destroy.argtypes = [vp]
        L.ref_set_state.argtypes = [vp, P(OrcGlobals), P(C.c_double), P(C.c_double)] + [P(C.c_int)] * 4
        L.ref_set_step.argtypes = [vp, C.c_uint64]
        L.ref_euler_step.argtypes = [vp, C.c_double, C.c_double]
        L.ref_get_state.argtypes = ([vp, P(OrcGlobals), P(C.c_double), P(C.c_double)] + [P(C.c_int)] * 4
                                    + [P(C.c_double)] * 3)
        L.ref_get_consts.argtypes = [vp, P(OrcConsts), P(OrcCurrents)]
        L.ref_cru_rates.argtypes = [P(OrcParams), C.c_double] + [P(C.c_int)] * 4 + [P(C.c_double)] * 6
        _ref = L
    return _ref


def default_params(**overrides) -> OrcParams:
    p = OrcParams()
    lib().orc_params_default(C.byref(p))
    for k, v in overrides.items():
        setattr(p, k, v)
    return p


def default_globals(py: bool = True) -> OrcGlobals:
    g = OrcGlobals()
    (lib().orc_globals_py_default if py else lib().orc_globals_default)(C.byref(g))
    return g


def constants(p: OrcParams, ncru: int) -> OrcConsts:
    c = OrcConsts()
    lib().orc_constants(C.byref(p), ncru, C.byref(c))
    return c


def uniforms(seed, cell, cru, step, n, umode=U53, stream=0, k0=0) -> np.ndarray:
    out = np.empty(n, dtype=np.float64)
    lib().orc_uniforms(seed, cell, cru, step, stream, umode, k0, n, _dp(out))
    return out


def philox(ctr, key) -> np.ndarray:
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().orc_philox4x32_10(c, k, o)
    return np.array(list(o), dtype=np.uint32)


class CRUArrays:
    """CRU state in the reference's layouts (pyGW.cpp:78-87)."""

    def __init__(self, n: int):
        self.n = n
        self.CaSS = np.zeros((n, 4))
        self.CaJSR = np.zeros(n)
        self.LCC = np.zeros((n, 4), dtype=np.int32)
        self.LCC_inactivation = np.zeros((n, 4), dtype=np.int32)
        self.RyR = np.zeros((n, 4, 6), dtype=np.int32)
        self.ClCh = np.zeros((n, 4), dtype=np.int32)

    def copy(self) -> "CRUArrays":
        o = CRUArrays(self.n)
        for k in ("CaSS", "CaJSR", "LCC", "LCC_inactivation", "RyR", "ClCh"):
            setattr(o, k, getattr(self, k).copy())
        return o

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k in ("CaSS", "CaJSR", "LCC", "LCC_inactivation", "RyR", "ClCh")}


class Model:
    """One cell in the C restatement (orc_model); timed=True uses the Release-flag build."""

    def __init__(self, p: OrcParams, ncru: int, seed: int = 0, cell: int = 0, umode: int = U53,
                 timed: bool = False):
        self.L = timed_lib() if timed else lib()
        self.n = ncru
        self.p = p
        self.h = self.L.orc_create(C.byref(p), ncru, seed, cell, umode)

    def __del__(self):
        if getattr(self, "h", None):
            self.L.orc_destroy(self.h)
            self.h = None

    def set_globals(self, g: OrcGlobals):
        self.L.orc_set_globals(self.h, C.byref(g))

    def globals(self) -> OrcGlobals:
        g = OrcGlobals()
        self.L.orc_get_globals(self.h, C.byref(g))
        return g

    def set_crus(self, s: CRUArrays):
        self.L.orc_set_crus(self.h, _dp(np.ascontiguousarray(s.CaSS, np.float64)),
                            _dp(np.ascontiguousarray(s.CaJSR, np.float64)),
                            _ip(np.ascontiguousarray(s.LCC, np.int32)),
                            _ip(np.ascontiguousarray(s.LCC_inactivation, np.int32)),
                            _ip(np.ascontiguousarray(s.RyR, np.int32)),
                            _ip(np.ascontiguousarray(s.ClCh, np.int32)))

    def crus(self) -> CRUArrays:
        s = CRUArrays(self.n)
        self.L.orc_get_crus(self.h, _dp(s.CaSS), _dp(s.CaJSR), _ip(s.LCC), _ip(s.LCC_inactivation),
                            _ip(s.RyR), _ip(s.ClCh))
        return s

    def set_fluxes(self, JLCC=None, Jxfer=None, Jtr=None):
        f = lambda a, shape: None if a is None else np.ascontiguousarray(a, np.float64).reshape(shape)
        a, b, c = f(JLCC, (self.n, 4)), f(Jxfer, (self.n, 4)), f(Jtr, (self.n,))
        self.L.orc_set_fluxes(self.h, _dp(a), _dp(b), _dp(c))

    def fluxes(self):
        JLCC = np.zeros((self.n, 4))
        Jxfer = np.zeros((self.n, 4))
        Jtr = np.zeros(self.n)
        self.L.orc_get_fluxes(self.h, _dp(JLCC), _dp(Jxfer), _dp(Jtr))
        return JLCC, Jxfer, Jtr

    def consts(self) -> OrcConsts:
        c = OrcConsts()
        self.L.orc_get_consts(self.h, C.byref(c))
        return c

    def currents(self) -> OrcCurrents:
        c = OrcCurrents()
        self.L.orc_get_currents(self.h, C.byref(c))
        return c

    def set_step(self, step: int):
        self.L.orc_set_step(self.h, step)

    def step_index(self) -> int:
        return int(self.L.orc_get_step(self.h))

    def sample_initial_crus(self):
        self.L.orc_sample_initial_crus(self.h)

    def euler_step(self, dt: float, Istim: float = 0.0):
        self.L.orc_euler_step(self.h, dt, Istim)

    def run(self, dt: float, istim: np.ndarray, record_every: int = 0):
        istim = np.ascontiguousarray(istim, dtype=np.float64)
        n = istim.size
        nrec = n // record_every if record_every > 0 else 0
        rec_t = np.zeros(max(nrec, 1))
        rec_g = (OrcGlobals * max(nrec, 1))()
        got = self.L.orc_run(self.h, dt, n, _dp(istim), record_every, nrec, _dp(rec_t), rec_g)
        G = np.frombuffer(bytes(rec_g), dtype=np.float64).reshape(-1, 36)[:got].copy()
        return rec_t[:got].copy(), G

    def run_record(self, dt: float, istim: np.ndarray, record_every: int, max_records=None):
        """run<PRNG> + record_state (pyGW.hpp:56-122): records after every step i with
        i % record_every == 0.  Returns (records the reference's loop makes, dict of the stored
        records: t [R], globals [R, 36] and the CRU arrays [R, n, ...]); R = max_records, by
        default num_steps // record_every, the reference's allocation (pyGW.hpp:109)."""
        istim = np.ascontiguousarray(istim, dtype=np.float64)
        n = self.n
        R = istim.size // record_every if max_records is None else int(max_records)
        Rb = max(R, 1)
        out = {"t": np.zeros(Rb), "CaSS": np.zeros((Rb, n, 4)), "CaJSR": np.zeros((Rb, n)),
               "LCC": np.zeros((Rb, n, 4), np.int32), "LCC_inactivation": np.zeros((Rb, n, 4), np.int32),
               "RyR": np.zeros((Rb, n, 4, 6), np.int32), "ClCh": np.zeros((Rb, n, 4), np.int32)}
        rec_g = (OrcGlobals * Rb)()
        made = self.L.orc_run_record(self.h, dt, istim.size, _dp(istim), record_every, R, _dp(out["t"]), rec_g,
                                     _dp(out["CaSS"]), _dp(out["CaJSR"]), _ip(out["LCC"]),
                                     _ip(out["LCC_inactivation"]), _ip(out["RyR"]), _ip(out["ClCh"]))
        out["globals"] = np.frombuffer(bytes(rec_g), dtype=np.float64).reshape(-1, 36).copy()
        k = min(int(made), R)
        return int(made), {key: v[:k] for key, v in out.items()}

    def events(self) -> int:
        return int(self.L.orc_event_count(self.h))


class RefModel:
    """One cell in the reference's own C++ (GW_model<double, InjectGen>)."""

    def __init__(self, p: OrcParams, ncru: int, seed: int = 0, cell: int = 0, umode: int = U53):
        self.L = ref_lib()
        self.n = ncru
        self.h = self.L.ref_create(C.byref(p), ncru, seed, cell, umode)

    def __del__(self):
        if getattr(self, "h", None):
            self.L.ref_destroy(self.h)
            self.h = None

    def set_state(self, g: OrcGlobals, s: CRUArrays):
        self.L.ref_set_state(self.h, C.byref(g), _dp(np.ascontiguousarray(s.CaSS, np.float64)),
                             _dp(np.ascontiguousarray(s.CaJSR, np.float64)),
                             _ip(np.ascontiguousarray(s.LCC, np.int32)),
                             _ip(np.ascontiguousarray(s.LCC_inactivation, np.int32)),
                             _ip(np.ascontiguousarray(s.RyR, np.int32)),
                             _ip(np.ascontiguousarray(s.ClCh, np.int32)))

    def set_step(self, step: int):
        self.L.ref_set_step(self.h, step)

    def euler_step(self, dt: float, Istim: float = 0.0):
        self.L.ref_euler_step(self.h, dt, Istim)

    def state(self):
        g = OrcGlobals()
        s = CRUArrays(self.n)
        JLCC = np.zeros((self.n, 4))
        Jxfer = np.zeros((self.n, 4))
        Jtr = np.zeros(self.n)
        self.L.ref_get_state(self.h, C.byref(g), _dp(s.CaSS), _dp(s.CaJSR), _ip(s.LCC),
                             _ip(s.LCC_inactivation), _ip(s.RyR), _ip(s.ClCh), _dp(JLCC),
                             _dp(Jxfer), _dp(Jtr))
        return g, s, (JLCC, Jxfer, Jtr)

    def consts(self):
        c = OrcConsts()
        cur = OrcCurrents()
        self.L.ref_get_consts(self.h, C.byref(c), C.byref(cur))
        return c, cur


def initial_crus(p: OrcParams, ncru: int, seed: int, cell: int = 0) -> CRUArrays:
    """The reference's random initial CRU distributions (GW_utils.tpp:5-64), counter-RNG keyed."""
    m = Model(p, ncru, seed=seed, cell=cell)
    m.sample_initial_crus()
    return m.crus()


def pulse_train(n: int, dt: float, amp: float, duration: float, period: float = 0.0,
                start: float = 0.0) -> np.ndarray:
    """Istim(t_i) with t accumulated by t += dt, as pyGW.hpp:110-116 does."""
    out = np.zeros(n)
    t = 0.0
    for i in range(n):
        tb = t - start
        if tb >= 0.0:
            if period > 0.0:
                tb = tb - period * float(int(tb / period))
            if tb < duration:
                out[i] = amp
        t += dt
    return out
