"""The FP32 screen of the FP64 SSA lane (SsaLane::surely_last in gw_kernel.cuh) through the C ABI's
diagnostic gw_screen_check.  The FP64 lanes (the FP64 engine and the gradient path) skip the FP64
rates of an iteration when the screen declares it the step's last; that is only sound if every
such iteration is one the FP64 iteration would also end the step with.

  cases        200,000 CRU states: LCC states 1-12, random inactivation gates and ClCh, the 5 RyRs
               of each subunit spread over the 6 states, some with the negative counts that the
               lumped 3/4 and 5/6 transitions leave (SSA.tpp:200-259); CaSS log-uniform over
               1e-6..2 and at and next to the regime thresholds 3.685e-2 and 1.15e-4
               (GW_utils.tpp:222-255); step values log-uniform over 1e-4..50 per ms
  pass 1       dt = inf: the FP64 iteration's jump time J of every case
  pass 2       dt = t + J (1 + eps) for eps from -1 to 1: the step ends before the jump for eps < 0
               (the iteration is the step's last) and after it for eps > 0.  The screen never
               declares an iteration last that the FP64 iteration is not (eps at and within ulps of
               0 included), and it declares at least 97 % of the cases with eps <= -1e-2 last (it
               declines where -log(u0) is within its margins, about 1e-4 absolute, of total (dt - t))
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 200_000
SEED = 77
EPS = np.array([-1.0, -0.5, -1e-2, -1e-3, -3e-4, -1e-4, -3e-5, -1e-5, -1e-6, -1e-9, -1e-13, 0.0, 1e-13, 1e-9,
                1e-6, 1e-4, 1e-2, 1.0])


def _cases(rng):
    lcc = rng.integers(1, 13, (N, 4)).astype(np.uint32)
    lcc_w = lcc[:, 0] | (lcc[:, 1] << 8) | (lcc[:, 2] << 16) | (lcc[:, 3] << 24)
    flags = rng.integers(0, 256, N).astype(np.uint32)
    counts = rng.multinomial(5, [1 / 6] * 6, (N, 4)).astype(np.int64)  # [case, subunit, state]
    neg = rng.random((N, 4)) < 0.05
    # lumped-regime leftovers: one state of a pair at -1, the other one above the pair's total
    for a, b in ((2, 3), (4, 5)):
        tot = counts[:, :, a] + counts[:, :, b]
        flip = neg & (rng.random((N, 4)) < 0.5)
        counts[:, :, a] = np.where(flip, -1, counts[:, :, a])
        counts[:, :, b] = np.where(flip, tot + 1, counts[:, :, b])
    planes = np.zeros((N, 6), dtype=np.uint32)
    for q in range(6):
        for j in range(4):
            planes[:, q] |= (counts[:, j, q].astype(np.int64) & 0xFF).astype(np.uint32) << (8 * j)
    chan = np.column_stack([lcc_w, flags, planes]).astype(np.uint32)
    cass = np.exp(rng.uniform(np.log(1e-6), np.log(2.0), (N, 4)))
    special = np.array([3.685e-2, np.nextafter(3.685e-2, 1), np.nextafter(3.685e-2, 0),
                        1.15e-4, np.nextafter(1.15e-4, 1), np.nextafter(1.15e-4, 0), 0.0])
    pick = rng.random((N, 4)) < 0.1
    cass = np.where(pick, special[rng.integers(0, special.size, (N, 4))], cass)
    sv = np.exp(rng.uniform(np.log(1e-4), np.log(50.0), (N, 40)))
    sv[:, 0] = 0.0
    t = np.where(rng.random(N) < 0.5, 0.0, rng.uniform(0.0, 1e-3, N))
    return np.ascontiguousarray(chan), np.ascontiguousarray(cass), np.ascontiguousarray(sv), t


def _run(L, p, chan, cass, sv, t, dt):
    from gwgb300 import _lib

    out = np.zeros((N, 2), dtype=np.int32)
    jump = np.zeros(N)
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    rc = L.gw_screen_check(C.byref(p), 12_500, N, chan.ctypes.data_as(C.POINTER(C.c_uint32)), dp(cass), dp(sv),
                           dp(t), dp(np.ascontiguousarray(dt)), SEED, out.ctypes.data_as(C.POINTER(C.c_int32)),
                           dp(jump))
    assert rc == _lib.GW_OK, _lib.last_error()
    return out[:, 0].astype(bool), out[:, 1].astype(bool), jump


def test_screen_is_sound_at_the_decision_boundary(enginelib):
    from gwgb300 import _lib

    L = _lib.load()
    p = _lib.default_params()
    rng = np.random.default_rng(SEED)
    chan, cass, sv, t = _cases(rng)
    sc, last, J = _run(L, p, chan, cass, sv, t, np.full(N, np.inf))
    assert not sc.any()  # an infinite step is never screened
    fin = ~last & np.isfinite(J) & (J > 0)
    assert fin.mean() > 0.9
    for eps in EPS:
        dt = np.where(fin, t + J * (1.0 + eps), 1e-3)
        sc, last, _ = _run(L, p, chan, cass, sv, t, dt)
        bad = sc & ~last
        assert not bad.any(), (eps, np.flatnonzero(bad)[:10])
        inside = fin & (t + J < dt)  # the jump lands inside the step (in FP64 arithmetic)
        assert not last[inside].any()
        if eps >= 1e-6:
            assert inside.sum() > 0.9 * fin.sum()
        if eps <= -1e-2:
            assert last[fin].all()
            assert sc[fin].mean() >= 0.97, (eps, sc[fin].mean())


def test_screen_passes_most_quiet_steps(enginelib):
    """CRUs near rest (RyRs closed, rates up to 2 per ms), dt = 1e-3 ms and t = 0: most draws give
    no event; the screen declares nearly all of those last, and none that has an event."""
    from gwgb300 import _lib

    L = _lib.load()
    p = _lib.default_params()
    rng = np.random.default_rng(SEED + 1)
    chan, cass, sv, _ = _cases(rng)
    chan[:, 2] = 0x05050505  # the 5 RyRs of every subunit closed (state 1), as at rest
    chan[:, 3:] = 0
    cass = np.exp(rng.uniform(np.log(1e-5), np.log(1e-2), (N, 4)))  # rest to early release
    sv = np.exp(rng.uniform(np.log(1e-3), np.log(2.0), (N, 40)))
    sv[:, 0] = 0.0
    t = np.zeros(N)
    sc, last, _ = _run(L, p, chan, cass, sv, t, np.full(N, 1e-3))
    assert not (sc & ~last).any()
    assert last.mean() > 0.5
    assert sc[last].mean() > 0.99, sc[last].mean()
