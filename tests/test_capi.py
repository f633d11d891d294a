"""The C-ABI library: it loads, exports every entry point include/gw_gb300.h declares, its struct
layouts match the ctypes bindings, its defaults match the reference's, and without a GPU it fails
cleanly (no compute calls here)."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import REPO

HEADER = os.path.join(REPO, "include", "gw_gb300.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:int|void)\s+(gw_\w+)\s*\(", src, flags=re.M)))


def test_exports_every_declared_symbol(enginelib):
    names = declared_functions()
    assert len(names) >= 20
    out = subprocess.run(["nm", "-D", "--defined-only", enginelib._name], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (gw_\w+)", out))
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    for n in names:
        assert hasattr(enginelib, n)


def test_status_codes_match_bindings():
    """Every gw_status the header declares has the same value in the Python mirror."""
    from gwgb300 import _lib

    src = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    body = re.search(r"typedef enum gw_status \{(.*?)\} gw_status;", src, flags=re.S).group(1)
    codes = dict((n, int(v)) for n, v in re.findall(r"(GW_\w+)\s*=\s*(\d+)", body))
    assert codes["GW_OK"] == 0 and "GW_ERR_SYNC_TIMEOUT" in codes
    for name, value in codes.items():
        assert getattr(_lib, name) == value, name


def test_struct_layouts_match_bindings(enginelib):
    from gwgb300 import _lib

    prog = r"""
#include <stdio.h>
#include <stddef.h>
#include "gw_gb300.h"
#define P(T) printf(#T " %zu\n", sizeof(T));
#define O(T, f) printf(#T "." #f " %zu\n", offsetof(T, f));
int main(void) {
  P(gw_params) P(gw_globals) P(gw_ensemble_desc) P(gw_trace) P(gw_stats) P(gw_grad_desc) P(gw_grad_stats)
  O(gw_params, NCaRU) O(gw_params, Ko) O(gw_params, Hr) O(gw_globals, Kr) O(gw_globals, Kv43)
  O(gw_globals, Kv14) O(gw_ensemble_desc, seed) O(gw_ensemble_desc, ode_fp32_rhs)
  O(gw_trace, cru_cell) O(gw_trace, n_written) O(gw_trace, cru_sums) O(gw_trace, CaJSR_f32)
  O(gw_trace, currents)
  O(gw_stats, kernel_ms) O(gw_stats, ctas) O(gw_stats, device_allocs)
  O(gw_grad_desc, seed) O(gw_grad_desc, dt) O(gw_grad_desc, n_steps) O(gw_grad_desc, stim)
  O(gw_grad_desc, event_cap) O(gw_grad_stats, events) O(gw_grad_stats, segment_bytes)
  return 0;
}
"""
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "l.c")
        exe = os.path.join(d, "l")
        open(src, "w").write(prog)
        subprocess.run(["gcc", "-I", os.path.dirname(HEADER), src, "-o", exe], check=True)
        lines = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split("\n")
    got = dict(l.split() for l in lines if l.strip())
    types = {"gw_params": _lib.GwParams, "gw_globals": _lib.GwGlobals, "gw_ensemble_desc": _lib.GwEnsembleDesc,
             "gw_trace": _lib.GwTrace, "gw_stats": _lib.GwStats, "gw_grad_desc": _lib.GwGradDesc,
             "gw_grad_stats": _lib.GwGradStats}
    for k, v in got.items():
        if "." in k:
            t, f = k.split(".")
            assert getattr(types[t], f).offset == int(v), k
        else:
            assert C.sizeof(types[k]) == int(v), k


def test_param_table_matches_reference_order(enginelib, oracle):
    from gwgb300 import _lib

    table = oracle.param_table()
    assert [n for _, n, _ in table] == _lib.PARAM_NAMES
    assert len(_lib.PARAM_NAMES) == 115
    p = _lib.default_params()
    for t, n, d in table:
        assert getattr(p, n) == (int(d) if t == "int" else d), n


def test_global_defaults(enginelib, oracle):
    from gwgb300 import _lib, engine

    g = engine.globals_to_array(_lib.default_globals())
    assert np.array_equal(g, oracle.default_globals(py=False).to_array())
    gp = engine.globals_to_array(_lib.default_globals(py=True))
    assert np.array_equal(gp, oracle.default_globals(py=True).to_array())
    assert gp[5] == 8.9282e-3 and g[5] == 8.98282e-3


def test_abi_version(enginelib):
    assert enginelib.gw_abi_version() == 5


def test_invalid_arguments_without_device(enginelib):
    from gwgb300 import _lib

    d = _lib.GwEnsembleDesc()
    h = C.c_void_p()
    assert enginelib.gw_create(None, C.byref(h)) == _lib.GW_ERR_INVALID_ARGUMENT
    d.n_cells = 0
    assert enginelib.gw_create(C.byref(d), C.byref(h)) == _lib.GW_ERR_INVALID_ARGUMENT
    assert "n_cells" in _lib.last_error()
    assert enginelib.gw_run(None, 1e-3, 10, 0, None) == _lib.GW_ERR_INVALID_ARGUMENT
    assert enginelib.gw_run_noalloc(None, 1e-3, 10, 0, None) == _lib.GW_ERR_INVALID_ARGUMENT
    assert enginelib.gw_autotune(None, 10, None, None, None) == _lib.GW_ERR_INVALID_ARGUMENT
    g = C.c_void_p()
    gd = _lib.GwGradDesc()
    assert enginelib.gw_grad_create(C.byref(gd), C.byref(g)) == _lib.GW_ERR_INVALID_ARGUMENT
    buf = C.create_string_buffer(256)
    enginelib.gw_grad_last_error(None, buf, len(buf))
    assert b"n_cells" in buf.value
    assert enginelib.gw_grad_forward(None, None) == _lib.GW_ERR_INVALID_ARGUMENT
    assert enginelib.gw_grad_backward(None, None, None) == _lib.GW_ERR_INVALID_ARGUMENT


def test_current_fields_match_bindings():
    from gwgb300 import _lib

    src = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    codes = dict((n, int(v)) for n, v in re.findall(r"(GW_CUR_\w+)\s*=\s*(\d+)", src))
    assert int(re.search(r"#define GW_CURRENTS (\d+)", src).group(1)) == len(_lib.CURRENT_FIELDS) == len(codes)
    for n, v in codes.items():
        assert _lib.CURRENT_FIELDS[v].upper() == n[len("GW_CUR_"):]


def test_grad_theta_enum_matches_bindings():
    from gwgb300 import _lib

    src = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    codes = dict((n, int(v)) for n, v in re.findall(r"(GW_TH_\w+)\s*=\s*(\d+)", src))
    assert sorted(codes.values()) == list(range(len(_lib.GRAD_THETA)))
    assert int(re.search(r"#define GW_GRAD_THETA (\d+)", src).group(1)) == len(_lib.GRAD_THETA)
    names = {"PCAL": "PCaL", "GKR": "GKr", "GKS": "GKs", "GK1": "GK1", "INAKMAX": "INaKmax", "VMAX": "Vmax",
             "RRYR": "rRyR", "CSQNT": "CSQNT"}
    for n, v in codes.items():
        assert _lib.GRAD_THETA[v] == names[n[len("GW_TH_"):]]


def test_unknown_prng_rejected_before_any_device_work(enginelib):
    from gwgb300 import _lib

    p = _lib.default_params()
    g = _lib.default_globals()
    rc = enginelib.gw_simulate(C.byref(p), 4, 1e-3, 10, None, 1, None, None, None, None, None, None,
                               C.byref(g), b"pcg64", 0, 0, None)
    assert rc == _lib.GW_ERR_INVALID_ARGUMENT
    assert _lib.last_error() == "pcg64"


def test_create_reports_missing_device_cleanly(enginelib):
    from gwgb300 import Ensemble, _lib

    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(_lib.GWError) as e:
        Ensemble([16])
    assert e.value.code == _lib.GW_ERR_NO_DEVICE


def test_cell_base_validated_without_device(enginelib):
    from gwgb300 import _lib

    d = _lib.GwEnsembleDesc()
    n = (C.c_int32 * 1)(16)
    p = _lib.default_params()
    d.n_cells, d.ncru, d.params = 1, n, C.pointer(p)
    h = C.c_void_p()
    for base in (-1, 1 << 28):
        d.cell_base = base
        assert enginelib.gw_create(C.byref(d), C.byref(h)) == _lib.GW_ERR_INVALID_ARGUMENT
        assert "cell_base" in _lib.last_error()
