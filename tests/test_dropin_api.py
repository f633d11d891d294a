"""The drop-in module GreensteinWinslow mirrors the reference's pybind11 surface (src/pyGW.cpp):
class names, fields, defaults, shapes, repr strings and errors.  Where the reference sources are
present, its own Python layer (src/model.py, src/parameters.py) is imported against this module."""
import numpy as np
import pytest


def test_parameters(GW, oracle):
    p = GW.GWParameters()
    assert repr(p) == "Greenstein and Winslow Model Parameters"
    for t, n, d in oracle.param_table():
        v = getattr(p, n)
        assert v == (int(d) if t == "int" else d)
        assert isinstance(v, int if t == "int" else float)
        setattr(p, n, v)
    assert "GKr" in dir(p)
    with pytest.raises(AttributeError):
        p.not_a_parameter = 1.0


def test_global_state(GW):
    g = GW.GWGlobalState()
    assert g.V == -91.382 and g.CaLTRPN == 8.9282e-3 and g.Cai == 1.45273e-4
    assert g.XKr.shape == (5,) and g.XKv14.shape == (10,) and g.XKv43.shape == (10,)
    assert g.XKv14[0] == 0.722328 and g.XKv43[0] == 0.953060
    g.XKr = np.ones(5)
    assert g.XKr.sum() == 5


def test_cru_state(GW):
    c = GW.GWCRUState(7)
    assert c.CaSS.shape == (7, 4) and c.CaSS.dtype == np.float64
    assert c.CaJSR.shape == (7,)
    assert c.LCC.shape == (7, 4) and c.LCC.dtype == np.int32
    assert c.RyR.shape == (7, 4, 6) and c.RyR.dtype == np.int32
    assert np.all(c.RyR.sum(axis=2) == 5)
    assert set(np.unique(c.LCC)) <= {1, 2, 7}
    c.ClCh = np.ones((7, 4))
    assert c.ClCh.dtype == np.int32
    with pytest.raises(ValueError):
        c.RyR = np.zeros((7, 4))


def test_variables(GW):
    v = GW.GWVariables(10, 3, 2.5)
    assert repr(v) == "Greenstein and Winslow model solution over the interval [0, 2.500000] with 10 CRUs"
    assert v.RyR.shape == (3, 10, 4, 6) and v.XKv14.shape == (3, 10) and v.CaSS.shape == (3, 10, 4)
    v.V = [1, 2, 3]
    assert v.V.dtype == np.float64


def test_run_rejects_unknown_prng(GW):
    with pytest.raises(ValueError):
        GW.run(GW.GWParameters(), 4, 1e-3, 10, lambda t: 0.0, 1, GW.GWCRUState(4), PRNG="pcg64")


def test_reference_python_layer_imports(ref_src, GW):
    params = ref_src.GWParameters(NCaRU_sim=64, GKr=0.03)
    assert isinstance(params.cxx_struct, GW.GWParameters)
    assert params.GKr == 0.03 and params.NCaRU_sim == 64
    d = params.to_dict()
    again = ref_src.GWParameters.from_dict(d)
    assert again.GKr == 0.03
    model = ref_src.GWModel(parameters=params, stimulus_fn=lambda t: 0.0)
    # run() raises ValueError as the pybind11 module does; src/model.py:974-978 then formats the
    # option list through a name-mangled class attribute and itself raises NameError (a defect of
    # the reference's Python layer, reproduced here unchanged).
    with pytest.raises((ValueError, NameError)) as e:
        model.simulate(1e-3, 10, PRNG="pcg64")
    assert isinstance(e.value, ValueError) or isinstance(e.value.__context__, ValueError)


def test_reference_solution_from_dict(ref_src, GW):
    n, R = 5, 3
    vars_ = {k: np.zeros(R) for k in ("t", "V", "Nai", "Ki", "Cai", "CaNSR", "CaLTRPN", "CaHTRPN", "m", "h", "j", "xKs")}
    vars_["t"] = np.array([0.1, 0.2, 0.3])
    vars_.update(XKr=np.zeros((R, 5)), XKv14=np.zeros((R, 10)), XKv43=np.zeros((R, 10)),
                 CaSS=np.zeros((R, n, 4)), CaJSR=np.zeros((R, n)), LCC=np.ones((R, n, 4), np.int32),
                 LCC_inactivation=np.ones((R, n, 4), np.int32), RyR=np.zeros((R, n, 4, 6), np.int32),
                 ClCh=np.zeros((R, n, 4), np.int32))
    params = ref_src.GWParameters(NCaRU_sim=n).to_dict()
    sol = ref_src.GWSolution.from_dict({"vars": vars_, "params": params})
    assert sol is not None
