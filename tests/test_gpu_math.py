"""The FP64 exp and log of the global step (table-driven, gw_math64.cuh) against the host's libm,
through the C ABI's diagnostic gw_math_check: within 2 units in the last place everywhere, and
exact where the result is exact (exp(0) = 1, log(2^k) = k ln2 rounded)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _check(x):
    from gwgb300 import _lib

    L = _lib.load()
    x = np.ascontiguousarray(x, dtype=np.float64)
    ex = np.empty_like(x)
    lg = np.empty_like(x)
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    assert L.gw_math_check(dp(x), x.size, dp(ex), dp(lg)) == _lib.GW_OK, _lib.last_error()
    return ex, lg


def _ulps(got, want):
    ok = np.isfinite(want) & (want != 0)
    return np.abs(got[ok] - want[ok]) / np.spacing(np.abs(want[ok]))


def test_exp_accuracy():
    rng = np.random.default_rng(1)
    x = np.concatenate([rng.uniform(-50, 50, 200_000),          # the global step's arguments
                        rng.uniform(-699.9, 699.9, 200_000),
                        rng.uniform(-1e-3, 1e-3, 50_000),
                        np.arange(-64, 65) * np.log(2) / 64,       # table boundaries
                        [0.0, -0.0, 1e-300, -1e-300, 699.99, -699.99]])
    ex, _ = _check(x)
    with np.errstate(over="ignore", under="ignore"):
        want = np.exp(x)
    u = _ulps(ex, want)
    assert u.max() <= 2.0, (u.max(), x[np.argmax(u)])
    assert np.all(ex[x == 0.0] == 1.0)


def test_exp_outside_the_table_range_falls_back():
    x = np.array([700.0, 709.0, 710.0, -720.0, -800.0, np.inf, -np.inf, np.nan])
    ex, _ = _check(x)
    with np.errstate(over="ignore", under="ignore"):
        want = np.exp(x)
    np.testing.assert_array_equal(np.isnan(ex), np.isnan(want))
    fin = np.isfinite(want) & (want > 0)
    assert np.all(np.abs(ex[fin] - want[fin]) <= 2 * np.spacing(want[fin]))
    assert ex[2] == np.inf and ex[5] == np.inf and ex[6] == 0.0


def test_log_accuracy():
    rng = np.random.default_rng(2)
    x = np.concatenate([rng.uniform(5.0, 20.0, 100_000),          # Nai
                        rng.uniform(100.0, 160.0, 100_000),        # Ki
                        np.exp(rng.uniform(-700, 700, 200_000)),
                        rng.uniform(0.9, 1.1, 50_000),            # the near-1 fallback and its edges
                        2.0 ** np.arange(-1020, 1020, 7),
                        [np.finfo(float).tiny, np.finfo(float).max, 0.96875, 1.03125, 0.96874999, 1.0312501]])
    _, lg = _check(x)
    want = np.log(x)
    u = _ulps(lg, want)
    assert u.max() <= 2.0, (u.max(), x[np.argmax(u)])
    assert lg[x == 1.0].tolist() == [0.0] * int(np.sum(x == 1.0))


def test_log_special_inputs():
    x = np.array([0.0, -0.0, -1.0, np.inf, np.nan, 5e-324, 1.0])
    _, lg = _check(x)
    with np.errstate(divide="ignore", invalid="ignore"):
        want = np.log(x)
    assert lg[0] == -np.inf and lg[1] == -np.inf
    assert np.isnan(lg[2]) and np.isnan(lg[4])
    assert lg[3] == np.inf
    assert abs(lg[5] - want[5]) <= 2 * np.spacing(abs(want[5]))
    assert lg[6] == 0.0
