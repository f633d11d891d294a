"""The gradient path on the GPU (gw_grad_*, gwgb300.adjoint).

  forward pass vs the oracle        3 cells of 64, 40 and 96 CRUs, 6,000 steps (a stimulated
                                    upstroke), V samples and final globals within 1e-12 relative
  replay at the recorded parameters bit-exact V (the frozen-trajectory replay reproduces the
                                    forward pass)
  adjoint vs central differences    4 cells x 500 CRUs x 20 ms after one stimulus, loss = MSE of V
                                    sampled every 0.5 ms against a target generated with the 8
                                    parameters scaled by 1 + U(-0.2, 0.2) (same seed: common random
                                    numbers); FD of frozen-trajectory replays with h = 1e-4 relative;
                                    rtol 1e-4, atol 1e-6 x the cell's largest sensitivity.  Where a
                                    +-h replay starts a different number of steps at V >= -40 mV
                                    than the recorded pass, the difference straddles the
                                    reference's discontinuous h/j gate rates (common.hpp:176-218)
                                    and measures the jump; h shrinks by 10 (to 1e-6) until it does
                                    not
  checkpoint interval               1,000 instead of 200: identical V and sensitivities
  torch.autograd.Function           gradient of the scales = sensitivities / scales
  heterogeneous cells               3 cells of 300, 180 and 420 CRUs, own parameter sets and stimulus
                                    times, 12 ms: adjoint vs central differences as above
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N_CELLS, NCRU, STEPS, SE, SEED = 4, 500, 20_000, 500, 31


def rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))


def test_forward_matches_oracle(oracle, enginelib):
    from gwgb300 import _lib
    from gwgb300.adjoint import GradEngine

    po = oracle
    ncru, steps, se, seed = [64, 40, 96], 6000, 500, 9
    p = po.default_params()
    gp = _lib.GwParams.from_buffer_copy(bytes(p))
    g0 = po.default_globals(py=True)
    states = [po.initial_crus(p, n, seed=seed, cell=c) for c, n in enumerate(ncru)]
    with GradEngine(ncru, gp, n_steps=steps, seed=seed, sample_every=se) as e:
        for c, s in enumerate(states):
            e.set_state(c, g0.to_array(), s)
        V = e.forward()
        G = [e.final_globals(c) for c in range(len(ncru))]
    istim = po.pulse_train(steps, 1e-3, 100.0, 0.5)
    for c, n in enumerate(ncru):
        m = po.Model(p, n, seed=seed, cell=c)
        m.set_globals(g0)
        m.set_crus(states[c])
        _, rec = m.run(1e-3, istim, record_every=1)
        Vo = rec[se - 1::se, 0]
        assert V.shape == (3, steps // se)
        assert rel(V[c], Vo) <= 1e-12
        assert rel(G[c], m.globals().to_array()) <= 1e-12
    assert V.max() > 0.0  # the stimulus fired an upstroke


@pytest.fixture(scope="module")
def recorded(enginelib):
    from gwgb300 import _lib
    from gwgb300.adjoint import THETA, GradEngine, initial_states, scaled_params

    base = _lib.default_params()
    g0 = np.frombuffer(bytes(_lib.default_globals(py=True)), dtype=np.float64).copy()
    states = initial_states([NCRU] * N_CELLS, seed=SEED)
    scales_t = 1.0 + np.random.default_rng(4).uniform(-0.2, 0.2, (N_CELLS, len(THETA)))
    kw = dict(n_steps=STEPS, seed=SEED, checkpoint_every=200, sample_every=SE)
    with GradEngine([NCRU] * N_CELLS, [scaled_params(base, s) for s in scales_t], **kw) as t:
        for c in range(N_CELLS):
            t.set_state(c, g0, states[c])
        Vt = t.forward()
    e = GradEngine([NCRU] * N_CELLS, base, **kw)
    for c in range(N_CELLS):
        e.set_state(c, g0, states[c])
    V = e.forward()
    dL = 2.0 * (V - Vt) / Vt.size
    sens = e.backward(dL)
    yield dict(e=e, base=base, g0=g0, states=states, Vt=Vt, V=V, dL=dL, sens=sens, kw=kw)
    e.close()


def test_recorded_pass_is_a_beat(recorded):
    V = recorded["V"]
    assert V.shape == (N_CELLS, STEPS // SE)
    assert V.max() > 0.0 and V[:, -1].max() < V.max()
    assert np.all(np.isfinite(recorded["sens"])) and np.all(np.abs(recorded["sens"]).max(axis=1) > 0)
    st = recorded["e"].stats()
    assert st["events"] > 0 and st["forward_ms"] > 0 and st["backward_ms"] > 0


def test_replay_at_recorded_parameters_is_bit_exact(recorded):
    e = recorded["e"]
    Vr, R = e.replay(list(range(N_CELLS)), [recorded["base"]] * N_CELLS, regime=True)
    np.testing.assert_array_equal(Vr, recorded["V"])
    np.testing.assert_array_equal(R, e.regime_steps())


def _loss_per_cell(V, Vt_rows, n_total):
    """Each cell's share of the loss mean((V - Vt)^2) over the whole target (n_total samples)."""
    return np.sum((V - Vt_rows) ** 2, axis=1) / n_total


def test_adjoint_matches_central_differences(recorded):
    from gwgb300.adjoint import THETA, scaled_params

    e, base, Vt, sens = recorded["e"], recorded["base"], recorded["Vt"], recorded["sens"]
    K = len(THETA)
    R0 = e.regime_steps()
    pairs = [(c, k) for c in range(N_CELLS) for k in range(K)]
    fd = np.full((N_CELLS, K), np.nan)
    used_h = np.zeros((N_CELLS, K))
    todo = pairs
    for h in (1e-4, 1e-5, 1e-6):
        src, params = [], []
        for c, k in todo:
            for sgn in (1.0, -1.0):
                s = np.ones(K)
                s[k] += sgn * h
                src.append(c)
                params.append(scaled_params(base, s))
        V, R = e.replay(src, params, regime=True)
        rows = Vt[np.asarray(src)]
        L = _loss_per_cell(V, rows, Vt.size)
        again = []
        for i, (c, k) in enumerate(todo):
            if R[2 * i] != R0[c] or R[2 * i + 1] != R0[c]:
                again.append((c, k))
                continue
            fd[c, k] = (L[2 * i] - L[2 * i + 1]) / (2 * h)
            used_h[c, k] = h
        todo = again
        if not todo:
            break
    assert not todo, f"every FD step straddles V = -40 mV for {todo}"
    for c in range(N_CELLS):
        np.testing.assert_allclose(sens[c], fd[c], rtol=1e-4, atol=1e-6 * np.max(np.abs(sens[c])),
                                   err_msg=f"cell {c}, FD steps {used_h[c]}")


def test_checkpoint_interval_does_not_change_results(recorded):
    from gwgb300.adjoint import GradEngine

    kw = dict(recorded["kw"], checkpoint_every=1000)
    with GradEngine([NCRU] * N_CELLS, recorded["base"], **kw) as e:
        for c in range(N_CELLS):
            e.set_state(c, recorded["g0"], recorded["states"][c])
        V = e.forward()
        sens = e.backward(recorded["dL"])
    np.testing.assert_array_equal(V, recorded["V"])
    np.testing.assert_array_equal(sens, recorded["sens"])


def test_autograd_function(recorded):
    import torch

    from gwgb300.adjoint import THETA, TraceSpec, VoltageTrace

    kw = recorded["kw"]
    spec = TraceSpec(ncru=[NCRU] * N_CELLS, base=recorded["base"],
                     states=[(recorded["g0"], s) for s in recorded["states"]], seed=kw["seed"],
                     n_steps=kw["n_steps"], checkpoint_every=kw["checkpoint_every"], sample_every=kw["sample_every"])
    scales = torch.ones(N_CELLS, len(THETA), dtype=torch.float64, requires_grad=True)
    V = VoltageTrace.apply(scales, spec)
    loss = torch.mean((V - torch.from_numpy(recorded["Vt"])) ** 2)
    loss.backward()
    np.testing.assert_array_equal(V.detach().numpy(), recorded["V"])
    np.testing.assert_allclose(scales.grad.numpy(), recorded["sens"], rtol=1e-12, atol=0)


def test_heterogeneous_cells_match_central_differences(enginelib):
    """Cells of 300, 180 and 420 CRUs with their own parameter sets (the 8 parameters scaled by
    1 + U(-0.15, 0.15)) and stimulus times (0, 1.5 and 3 ms), 12 ms: every relative sensitivity of
    every cell against central differences of frozen-trajectory replays (h = 1e-4, smaller where a
    +-h replay starts a different number of steps at V >= -40 mV), rtol 1e-4."""
    from gwgb300 import _lib
    from gwgb300.adjoint import THETA, GradEngine, initial_states, scaled_params

    ncru, steps, se, seed = [300, 180, 420], 12_000, 250, 5
    base = _lib.default_params()
    rng = np.random.default_rng(8)
    pscale = 1.0 + rng.uniform(-0.15, 0.15, (3, len(THETA)))
    params = [scaled_params(base, pscale[c]) for c in range(3)]
    stim = np.array([[0.0, 0.0, 0.5, 100.0], [1.5, 0.0, 0.5, 100.0], [3.0, 0.0, 0.5, 100.0]])
    g0 = np.frombuffer(bytes(_lib.default_globals(py=True)), dtype=np.float64).copy()
    states = initial_states(ncru, seed=seed)
    kw = dict(n_steps=steps, seed=seed, checkpoint_every=300, sample_every=se, stim=stim)
    tscale = 1.0 + rng.uniform(-0.2, 0.2, (3, len(THETA)))
    with GradEngine(ncru, [scaled_params(params[c], tscale[c]) for c in range(3)], **kw) as t:
        for c in range(3):
            t.set_state(c, g0, states[c])
        Vt = t.forward()
    with GradEngine(ncru, params, **kw) as e:
        for c in range(3):
            e.set_state(c, g0, states[c])
        V = e.forward()
        sens = e.backward(2.0 * (V - Vt) / Vt.size)
        R0 = e.regime_steps()
        K = len(THETA)
        fd = np.full((3, K), np.nan)
        todo = [(c, k) for c in range(3) for k in range(K)]
        for h in (1e-4, 1e-5, 1e-6):
            src, pv = [], []
            for c, k in todo:
                for sgn in (1.0, -1.0):
                    s = np.ones(K)
                    s[k] += sgn * h
                    src.append(c)
                    pv.append(scaled_params(params[c], s))
            Vr, R = e.replay(src, pv, regime=True)
            L = np.sum((Vr - Vt[np.asarray(src)]) ** 2, axis=1) / Vt.size
            again = []
            for i, (c, k) in enumerate(todo):
                if R[2 * i] != R0[c] or R[2 * i + 1] != R0[c]:
                    again.append((c, k))
                else:
                    fd[c, k] = (L[2 * i] - L[2 * i + 1]) / (2 * h)
            todo = again
            if not todo:
                break
    assert not todo, todo
    assert V.max() > 0.0 and np.all(V[:, -1] > V[:, 0])  # every cell fired
    for c in range(3):
        np.testing.assert_allclose(sens[c], fd[c], rtol=1e-4, atol=1e-6 * np.max(np.abs(sens[c])), err_msg=f"cell {c}")
