"""gw_run_noalloc through the C ABI: the variant of gw_run that stages its records in a static
device array instead of allocating.  On two calls in a row it must give gw_run's records and
state, also when its scratch forces shorter launches than gw_run's, and it must reject a trace
whose records cannot fit the scratch.  (File name sorts last so it also runs after the rest.)"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ("CaSS", "CaJSR", "LCC", "LCC_inactivation", "RyR", "ClCh")


def _trace(n_cells, nrec, ncru, cru_cell, fields=FIELDS):
    from gwgb300 import _lib

    tr = _lib.GwTrace()
    tr.max_records = nrec
    arrs = {"t": np.zeros(nrec), "globals": np.zeros((n_cells, nrec, 36))}
    tr.t = arrs["t"].ctypes.data_as(C.POINTER(C.c_double))
    tr.globals = arrs["globals"].ctypes.data_as(C.POINTER(C.c_double))
    tr.cru_cell = cru_cell
    shapes = {"CaSS": ((nrec, ncru, 4), np.float64), "CaJSR": ((nrec, ncru), np.float64),
              "LCC": ((nrec, ncru, 4), np.int32), "LCC_inactivation": ((nrec, ncru, 4), np.int32),
              "RyR": ((nrec, ncru, 4, 6), np.int32), "ClCh": ((nrec, ncru, 4), np.int32)}
    for f in fields:
        shape, dt = shapes[f]
        arrs[f] = np.full(shape, -7, dtype=dt)  # not zero: every element must be written
        ct = C.c_double if dt == np.float64 else C.c_int32
        setattr(tr, f, arrs[f].ctypes.data_as(C.POINTER(ct)))
    return tr, arrs


def _ensemble(ncru, precision, seed):
    from gwgb300 import Ensemble

    e = Ensemble(ncru, precision=precision, seed=seed)
    for c in range(len(ncru)):
        e.sample_initial_crus(c)
    e.set_pulse(0.0, 1000.0, 0.5, 100.0)
    return e


def _run(e, fn, dt, n, every, cru_cell):
    from gwgb300 import _lib

    nrec = n // every
    tr, arrs = _trace(e.n_cells, nrec, int(e.ncru[cru_cell]), cru_cell)
    rc = getattr(e.L, fn)(e.h, dt, n, every, C.byref(tr))
    assert rc == _lib.GW_OK, (fn, rc, _lib.last_error(e.h))
    assert tr.n_written == nrec
    return arrs


def _same(ra, rb):
    # the same engine launches on the same state and draws: bit for bit the same records
    assert ra.keys() == rb.keys()
    for k in ra:
        assert np.array_equal(ra[k], rb[k]), k


def _state(e, cell=0):
    s = e.get_crus(cell)
    return e.get_globals(cell), s


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_noalloc_matches_gw_run_on_two_calls(precision):
    ncru = [1500, 700]
    a = _ensemble(ncru, precision, seed=21)
    b = _ensemble(ncru, precision, seed=21)
    for call in range(2):
        ra = _run(a, "gw_run", 1e-3, 400, 40, cru_cell=1)
        rb = _run(b, "gw_run_noalloc", 1e-3, 400, 40, cru_cell=1)
        _same(ra, rb)
        assert np.all(ra["LCC"] >= 1) and np.all(ra["LCC"] <= 12)
        ga, sa = _state(a)
        gb, sb = _state(b)
        assert np.array_equal(gb, ga)
        for f in ("CaSS", "CaJSR", "JLCC", "LCC", "LCC_inactivation", "RyR", "ClCh"):
            assert np.array_equal(getattr(sa, f), getattr(sb, f)), (call, f)
        assert a.time(0) == b.time(0)
    a.close()
    b.close()


def test_noalloc_allocates_no_device_memory():
    """After its first call on a device, gw_run_noalloc makes no cudaMalloc (the library counts
    every one it makes, gw_stats.device_allocs); gw_run, for comparison, allocates its record
    staging on every call."""
    e = _ensemble([1500, 700], "fp64", seed=8)
    _run(e, "gw_run_noalloc", 1e-3, 200, 40, cru_cell=1)
    n0 = e.stats()["device_allocs"]
    for _ in range(2):
        _run(e, "gw_run_noalloc", 1e-3, 200, 40, cru_cell=1)
    assert e.stats()["device_allocs"] == n0
    _run(e, "gw_run", 1e-3, 200, 40, cru_cell=1)
    assert e.stats()["device_allocs"] > n0
    e.close()


def test_noalloc_shortens_launches_to_fit_its_scratch():
    # 12,500 CRUs with every CRU field: about 3 MB of staging per record, so the 16 MiB scratch
    # holds 5 records and the launches of 1000 steps at 100 steps per record are cut to 250.
    a = _ensemble([12500], "fp32", seed=5)
    b = _ensemble([12500], "fp32", seed=5)
    for call in range(2):
        ra = _run(a, "gw_run", 1e-3, 600, 100, cru_cell=0)
        rb = _run(b, "gw_run_noalloc", 1e-3, 600, 100, cru_cell=0)
        _same(ra, rb)
    assert b.stats()["launches"] > a.stats()["launches"]
    a.close()
    b.close()


def test_noalloc_rejects_records_beyond_its_scratch():
    from gwgb300 import _lib

    e = _ensemble([30000], "fp32", seed=3)
    tr, _ = _trace(1, 4, 30000, 0)
    rc = e.L.gw_run_noalloc(e.h, 1e-3, 40, 10, C.byref(tr))
    assert rc == _lib.GW_ERR_INVALID_ARGUMENT
    msg = _lib.last_error(e.h)
    assert "scratch" in msg and "gw_run" in msg
    # the same context still runs without a trace and with globals-only records
    assert e.L.gw_run_noalloc(e.h, 1e-3, 20, 0, None) == _lib.GW_OK
    tr2, arrs = _trace(1, 2, 30000, -1, fields=())
    assert e.L.gw_run_noalloc(e.h, 1e-3, 20, 10, C.byref(tr2)) == _lib.GW_OK
    assert tr2.n_written == 2 and np.all(np.isfinite(arrs["globals"]))
    e.close()
