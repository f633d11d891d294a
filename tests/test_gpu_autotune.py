"""gw_autotune: picks a cluster size and CTA capacity that fit the cells, reports its time per
step, and the ensemble built with them runs (through the C ABI and through
Ensemble(cluster_ctas="auto"))."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _desc(ncru, keep):
    from gwgb300 import _lib

    n = np.ascontiguousarray(ncru, dtype=np.int32)
    p = (_lib.GwParams * 1)(_lib.default_params())
    d = _lib.GwEnsembleDesc()
    d.n_cells = n.size
    d.ncru = n.ctypes.data_as(C.POINTER(C.c_int32))
    d.params = C.cast(p, C.POINTER(_lib.GwParams))
    d.precision = _lib.PRECISION["fp32"]
    d.seed = 5
    keep += [n, p]
    return d


@pytest.mark.parametrize("ncru,allowed", [([12500], {6, 8, 9, 16}), ([300] * 6, {1, 2, 3, 4, 6, 8, 9, 16})])
def test_autotune_picks_a_fitting_shape(ncru, allowed):
    from gwgb300 import _lib

    L = _lib.load()
    keep = []
    d = _desc(ncru, keep)
    best, tile, us = C.c_int(), C.c_int(-1), C.c_double()
    assert L.gw_autotune(C.byref(d), 100, C.byref(best), C.byref(tile), C.byref(us)) == _lib.GW_OK, _lib.last_error()
    assert best.value in allowed and 0.0 < us.value < 1e4
    assert tile.value == 0 or tile.value >= 64
    d.cluster_ctas = best.value
    d.cta_crus = tile.value
    h = C.c_void_p()
    assert L.gw_create(C.byref(d), C.byref(h)) == _lib.GW_OK
    assert L.gw_run(h, 1e-3, 50, 0, None) == _lib.GW_OK
    L.gw_destroy(h)


def test_ensemble_auto_shape():
    from gwgb300 import Ensemble

    e = Ensemble([3000, 2000, 1200], precision="fp32", seed=3, cluster_ctas="auto", tune_steps=60)
    assert e.tuned_us_per_step > 0
    for c in range(3):
        e.sample_initial_crus(c)
    tr = e.run(1e-3, 100, record_every=50)
    assert np.all(np.isfinite(tr.globals))
    assert e.stats()["cluster_ctas"] in (1, 2, 3, 4, 6, 8, 9, 16)
    e.close()


def test_autotune_tile_optional_and_uneven_cells():
    """best_cta_crus may be NULL; for uneven cells the chosen capacity fits them all."""
    from gwgb300 import _lib

    L = _lib.load()
    keep = []
    d = _desc([4000, 1500, 2600, 900], keep)
    best, us = C.c_int(), C.c_double()
    assert L.gw_autotune(C.byref(d), 60, C.byref(best), None, C.byref(us)) == _lib.GW_OK, _lib.last_error()
    assert best.value in (1, 2, 3, 4, 6, 8, 9, 16) and us.value > 0.0
