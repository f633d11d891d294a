"""Failure detection on the GPU without a GPU fault: the kernel records the first error of each
cell in a status word, finishes its launch, and gw_run returns the status; the context stays
usable afterwards.  The failures are made on the host (a jump cap of 1, a negative concentration,
a NaN voltage), never by a bad address or a trap."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cell(**kw):
    from gwgb300 import Ensemble

    e = Ensemble([300], precision=kw.pop("precision", "fp32"), seed=9, **kw)
    e.sample_initial_crus(0)
    e.set_pulse(0.0, 1000.0, 0.5, 100.0)
    return e


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_event_cap(precision):
    from gwgb300 import _lib

    e = _cell(precision=precision, event_cap=1)
    with pytest.raises(_lib.GWError) as ex:
        e.run(1e-3, 3000)  # the AP's release makes some CRU jump more than once in a step
    assert ex.value.code == _lib.GW_ERR_EVENT_CAP
    assert "jump cap" in str(ex.value)
    # the context still answers and runs
    g = e.get_globals(0)
    assert np.all(np.isfinite(g))
    e.close()


def test_nernst_argument():
    from gwgb300 import _lib

    e = _cell()
    ck = e.checkpoint(0)
    g = e.get_globals(0)
    g[1] = -1.0  # Nai <= 0: the reference calls exit() here (common.hpp:72-75)
    e.set_globals(0, g)
    with pytest.raises(_lib.GWError) as ex:
        e.run(1e-3, 5)
    assert ex.value.code == _lib.GW_ERR_NERNST
    e.restore(0, ck)
    e.run(1e-3, 5)  # usable again from a good state
    assert np.all(np.isfinite(e.get_globals(0)))
    e.close()


def test_nonfinite_global():
    from gwgb300 import _lib

    e = _cell()
    g = e.get_globals(0)
    g[0] = np.nan
    e.set_globals(0, g)
    with pytest.raises(_lib.GWError) as ex:
        e.run(1e-3, 5)
    assert ex.value.code == _lib.GW_ERR_NONFINITE
    e.close()


def test_errors_are_per_cell():
    """One failing cell does not stop the others: their globals advance normally."""
    from gwgb300 import Ensemble, _lib

    e = Ensemble([300, 300], precision="fp32", seed=9)
    for c in range(2):
        e.sample_initial_crus(c)
    g = e.get_globals(1)
    g[2] = 0.0  # Ki = 0 in cell 1
    e.set_globals(1, g)
    g0 = e.get_globals(0).copy()
    with pytest.raises(_lib.GWError) as ex:
        e.run(1e-3, 10)
    assert ex.value.code == _lib.GW_ERR_NERNST and "cell 1" in str(ex.value)
    assert np.all(np.isfinite(e.get_globals(0))) and not np.array_equal(e.get_globals(0), g0)
    e.close()


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_bounded_wait_runs_out(monkeypatch, precision):
    """The per-step data travel by st.async on mbarriers whose waits are bounded.  The test hook
    makes the last wait of each launch expect 16 bytes that no one sends (a flag nothing sets):
    the wait runs out after about a second, the launch finishes, the run reports
    GW_ERR_SYNC_TIMEOUT, and the context answers; a context made without the hook runs normally."""
    from gwgb300 import _lib

    monkeypatch.setenv("GWGB300_TEST_SYNC_TIMEOUT", "1")
    e = _cell(precision=precision, steps_per_launch=20)
    with pytest.raises(_lib.GWError) as ex:
        e.run(1e-3, 20)  # one launch: its final wait runs out
    assert ex.value.code == _lib.GW_ERR_SYNC_TIMEOUT
    assert "bounded wait" in str(ex.value)
    assert np.all(np.isfinite(e.get_globals(0)))
    e.close()
    monkeypatch.delenv("GWGB300_TEST_SYNC_TIMEOUT")
    f = _cell(precision=precision, steps_per_launch=20)
    f.run(1e-3, 40)
    assert np.all(np.isfinite(f.get_globals(0)))
    f.close()
