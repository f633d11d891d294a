"""Oracle restatement vs the reference's own C++ (only where oracle/_ref was built from the
reference sources): random seeds, parameters and initial states, bit for bit."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def ref(oracle):
    if not oracle.ref_available():
        pytest.skip("reference harness not built here")
    return oracle


@pytest.mark.parametrize("seed", [1, 2, 3])
@pytest.mark.parametrize("umode", [0, 1])
def test_bit_exact(ref, seed, umode):
    po = ref
    rng = np.random.default_rng(seed)
    over = {"PCaL": 9.13e-13 * rng.uniform(0.8, 1.5), "rRyR": 3.92 * rng.uniform(0.8, 1.3),
            "NCaRU": int(rng.integers(2000, 20000))}
    p = po.default_params(**over)
    n = int(rng.integers(8, 40))
    init = po.initial_crus(p, n, seed=seed + 7)
    g0 = po.default_globals(py=True)
    steps = 2500
    istim = po.pulse_train(steps, 1e-3, 100.0, 0.5)
    m = po.Model(p, n, seed=seed, umode=umode)
    m.set_globals(g0)
    m.set_crus(init)
    r = po.RefModel(p, n, seed=seed, umode=umode)
    r.set_state(g0, init)
    for i in range(steps):
        m.euler_step(1e-3, istim[i])
        r.euler_step(1e-3, istim[i])
    g, s, fl = r.state()
    assert np.array_equal(m.globals().to_array(), g.to_array())
    sm = m.crus()
    for k in ("CaSS", "CaJSR", "LCC", "LCC_inactivation", "RyR", "ClCh"):
        assert np.array_equal(getattr(sm, k), getattr(s, k)), k
    for a, b in zip(m.fluxes(), fl):
        assert np.array_equal(a, b)


def test_open_lcc_initial_state(ref):
    """An initial state with open LCCs: the reference's ctor computes JLCC from its own random CRU
    state (GW.hpp:104-112, states 1, 2 or 7, so JLCC = 0) before set_initial_value installs this one;
    the oracle starts from JLCC = 0 too, and both runs agree bit for bit, JLCC included."""
    po = ref
    n, steps = 30, 400
    p = po.default_params()
    init = po.initial_crus(p, n, seed=3)
    rng = np.random.default_rng(3)
    pick = rng.random((n, 4)) < 0.3
    init.LCC[pick] = rng.choice([6, 12], size=int(pick.sum()))
    init.LCC_inactivation[pick] = 1
    g0 = po.default_globals(py=True)
    m = po.Model(p, n, seed=4)
    m.set_globals(g0)
    m.set_crus(init)
    r = po.RefModel(p, n, seed=4)
    r.set_state(g0, init)
    assert not np.any(r.state()[2][0])  # the ctor's JLCC, before any step
    istim = po.pulse_train(steps, 1e-3, 100.0, 0.5)
    for i in range(steps):
        m.euler_step(1e-3, istim[i])
        r.euler_step(1e-3, istim[i])
    g, s, fl = r.state()
    assert np.array_equal(m.globals().to_array(), g.to_array())
    for k in ("CaSS", "CaJSR", "LCC", "LCC_inactivation", "RyR", "ClCh"):
        assert np.array_equal(getattr(m.crus(), k), getattr(s, k)), k
    for a, b in zip(m.fluxes(), fl):
        assert np.array_equal(a, b)
