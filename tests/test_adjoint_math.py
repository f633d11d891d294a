"""The hand-written adjoints of the gradient path (gw_adjoint_math.h), on the host.

gw_grad_check_global evaluates one global increment (update_V_and_concentration_derivatives,
update_gate_derivatives, the IKr and Kv chains: GW.tpp:26-212) and its adjoint; gw_grad_check_cru
one CRU step of given sub-steps and events (update_fluxes SSA.tpp:37-45, update_CaSS :87-99,
update_CaJSR SSA.hpp:68-71, JLCC and Jrel at transitions :103-283) and its adjoint.

  increment vs the oracle's euler_step      G + d within 1e-14 relative, at states along a beat
  adjoints vs central differences           of lam . d (global) and lam . x_out + lam_c . carry (CRU),
                                            rtol 1e-4 with atol 1e-6 x the largest entry for the
                                            global step (FD steps of 1e-4 relative), rtol 1e-5 for
                                            the CRU's states and inputs, 1e-4 for rRyR and CSQNT
No device: the library is loaded and these two entry points run on the CPU.
"""
import ctypes as C

import numpy as np
import pytest

DT = 1e-3
THETA_FIELDS = (("PCaL",), ("GKr",), ("GKs",), ("GK1",), ("INaKmax",), ("Vmaxf", "Vmaxr"), ("rRyR",), ("CSQNT",))
PICKS = (0, 150, 400, 2000, 8000, 30000, 59000)  # rest, upstroke, peak, early plateau, plateau, repolarised


def dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


@pytest.fixture(scope="module")
def lib(enginelib):
    return enginelib


@pytest.fixture(scope="module")
def beat_states(oracle):
    """(globals, carry, Istim, globals after the oracle's euler_step) at PICKS of a 50-CRU beat."""
    po = oracle
    p = po.default_params()
    n = 50
    m = po.Model(p, n, seed=3)
    m.set_globals(po.default_globals(py=True))
    m.set_crus(po.initial_crus(p, n, seed=3))
    istim = po.pulse_train(max(PICKS) + 1, DT, 100.0, 0.5)
    out, i = [], 0
    for k in PICKS:
        if k > i:
            m.run(DT, istim[i:k])
        g = m.globals().to_array()
        JLCC, Jxfer, Jtr = m.fluxes()
        carry = np.array([JLCC.sum(), m.crus().ClCh.sum(), Jtr.sum(), Jxfer.sum()], float)
        m.euler_step(DT, istim[k])
        out.append((g, carry, float(istim[k]), m.globals().to_array()))
        i = k + 1
    return p, out


def gparams(p, **scale):
    from gwgb300 import _lib

    q = _lib.GwParams.from_buffer_copy(bytes(p))
    for k, s in scale.items():
        setattr(q, k, getattr(q, k) * s)
    return q


def increment(lib, p, g, carry, istim, lam):
    d, lg, lc, lt = np.zeros(36), np.zeros(36), np.zeros(3), np.zeros(8)
    rc = lib.gw_grad_check_global(C.byref(p), 50, dp(np.ascontiguousarray(g)), dp(np.ascontiguousarray(carry)),
                                  istim, DT, dp(lam), dp(d), dp(lg), dp(lc), dp(lt))
    assert rc == 0
    return d, lg, lc, lt


def test_global_increment_matches_oracle(lib, beat_states):
    p, states = beat_states
    gp = gparams(p)
    V = [s[0][0] for s in states]
    assert max(V) > 0.0 and min(V) < -80.0  # the picks span rest and the upstroke
    for g, carry, istim, g_new in states:
        d, *_ = increment(lib, gp, g, carry, istim, np.zeros(36))
        assert np.max(np.abs((g + d) - g_new) / np.maximum(np.abs(g_new), 1e-300)) <= 1e-14


def test_global_adjoint_vs_central_differences(lib, beat_states):
    p, states = beat_states
    gp = gparams(p)
    rng = np.random.default_rng(11)
    for g, carry, istim, _ in states:
        lam = rng.standard_normal(36)
        _, lg, lc, lt = increment(lib, gp, g, carry, istim, lam)

        def J(gg=g, cc=carry, pp=gp):
            return float(lam @ increment(lib, pp, gg, cc, istim, np.zeros(36))[0])

        fd = np.zeros(36)
        for k in range(36):
            h = 1e-4 * max(abs(g[k]), 1e-3 if k >= 7 else 0.0) + 1e-14
            gp_, gm_ = g.copy(), g.copy()
            gp_[k] += h
            gm_[k] -= h
            fd[k] = (J(gg=gp_) - J(gg=gm_)) / (2 * h)
        adj = lg - lam
        np.testing.assert_allclose(adj, fd, rtol=1e-4, atol=1e-6 * np.max(np.abs(adj)))
        # carry sums JLCC, Jtr, Jxfer (carry indices 0, 2, 3)
        fdc = np.zeros(3)
        for q, k in enumerate((0, 2, 3)):
            h = 1e-3 * abs(carry[k]) + 1e-3
            cp_, cm_ = carry.copy(), carry.copy()
            cp_[k] += h
            cm_[k] -= h
            fdc[q] = (J(cc=cp_) - J(cc=cm_)) / (2 * h)
        np.testing.assert_allclose(lc, fdc, rtol=1e-4, atol=1e-9 * np.max(np.abs(lc)))
        # relative sensitivities of the global-step parameters
        fdt = np.zeros(8)
        for k in (1, 2, 3, 4, 5):
            h = 1e-3
            up = gparams(p, **{f: 1 + h for f in THETA_FIELDS[k]})
            dn = gparams(p, **{f: 1 - h for f in THETA_FIELDS[k]})
            fdt[k] = (J(pp=up) - J(pp=dn)) / (2 * h)
        assert lt[0] == 0.0 and lt[6] == 0.0 and lt[7] == 0.0
        np.testing.assert_allclose(lt, fdt, rtol=1e-4, atol=1e-6 * np.max(np.abs(lt)))


def cru_case(oracle, n_sub, seed):
    po = oracle
    p = po.default_params()
    rng = np.random.default_rng(seed)
    x = np.concatenate([10.0 ** rng.uniform(-4, -1.5, 4), [rng.uniform(0.3, 1.0)], rng.uniform(0, 0.5, 4)])
    x[5 + rng.integers(0, 4)] = 0.0  # a non-conducting subunit
    o = rng.integers(0, 6, 4).astype(np.int32)
    V = rng.uniform(-60, 30)
    c = po.constants(p, 50)
    e = np.exp(-V * c.F_RT)
    JE = (1.0 / e) ** 2
    JM = c.JLCC_const * V * c.F_RT / (JE - 1)
    cin = np.array([10.0 ** rng.uniform(-4, -3), rng.uniform(0.5, 1.5), JM, JE])
    h = rng.dirichlet(np.ones(n_sub)) * DT * rng.uniform(0.5, 1.0)
    ev = rng.integers(0, 4, n_sub).astype(np.int32)
    ev[-1] = 0  # the step's last sub-step ends at the end of the step, with no event
    sub = rng.integers(0, 4, n_sub).astype(np.int32)
    onew = rng.integers(0, 6, n_sub).astype(np.int32)
    return p, x, o, cin, h, ev, sub, onew


def cru_run(lib, p, x, o, cin, h, ev, sub, onew, lx, lcar):
    xo, co, lx0, lin, lpar = np.zeros(9), np.zeros(2), np.zeros(9), np.zeros(4), np.zeros(2)
    rc = lib.gw_grad_check_cru(C.byref(p), 50, dp(np.ascontiguousarray(x)), ip(o), dp(np.ascontiguousarray(cin)),
                               int(h.size), dp(h), ip(ev), ip(sub), ip(onew), dp(lx), dp(lcar), dp(xo), dp(co),
                               dp(lx0), dp(lin), dp(lpar))
    assert rc == 0
    return xo, co, lx0, lin, lpar


@pytest.mark.parametrize("n_sub,seed", [(1, 1), (2, 2), (5, 3), (17, 4), (17, 5)])
def test_cru_adjoint_vs_central_differences(oracle, lib, n_sub, seed):
    p, x, o, cin, h, ev, sub, onew = cru_case(oracle, n_sub, seed)
    gp = gparams(p)
    rng = np.random.default_rng(100 + seed)
    lx, lcar = rng.standard_normal(9), rng.standard_normal(2)
    _, _, lx0, lin, lpar = cru_run(lib, gp, x, o, cin, h, ev, sub, onew, lx, lcar)

    def J(xx=x, cc=cin, pp=gp):
        xo, co, *_ = cru_run(lib, pp, xx, o, cc, h, ev, sub, onew, np.zeros(9), np.zeros(2))
        return float(lx @ xo + lcar @ co)

    fdx = np.zeros(9)
    for k in range(9):
        hk = 1e-4 * max(abs(x[k]), 1e-4)
        a, b = x.copy(), x.copy()
        a[k] += hk
        b[k] -= hk
        fdx[k] = (J(xx=a) - J(xx=b)) / (2 * hk)
    np.testing.assert_allclose(lx0, fdx, rtol=1e-5, atol=1e-9 * np.max(np.abs(lx0)))
    fdi = np.zeros(4)
    for k in range(4):
        hk = 1e-4 * abs(cin[k])
        a, b = cin.copy(), cin.copy()
        a[k] += hk
        b[k] -= hk
        fdi[k] = (J(cc=a) - J(cc=b)) / (2 * hk)
    np.testing.assert_allclose(lin, fdi, rtol=1e-5, atol=1e-9 * np.max(np.abs(lin)))
    # rRyR (relative) and CSQNT: dL/dCSQN_const with CSQN_const = KCSQN * CSQNT
    hr = 1e-3
    fd_r = (J(pp=gparams(p, rRyR=1 + hr)) - J(pp=gparams(p, rRyR=1 - hr))) / (2 * hr)
    fd_c = (J(pp=gparams(p, CSQNT=1 + hr)) - J(pp=gparams(p, CSQNT=1 - hr))) / (2 * hr)
    scale = 1.0 + abs(lx @ np.concatenate([x[:5], x[5:]]))
    assert abs(lpar[0] - fd_r) <= 1e-4 * max(abs(fd_r), 1e-6 * scale)
    assert abs(lpar[1] * p.KCSQN * p.CSQNT - fd_c) <= 1e-4 * max(abs(fd_c), 1e-6 * scale)
