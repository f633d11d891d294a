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
