import importlib
import os
import sys
import types

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(REPO, "gw-model_gb300"), os.path.join(REPO, "oracle"), REPO):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(REPO, "tests", "golden")


def _reference_dir():
    import pyoracle

    return pyoracle.reference_dir()


# the reference checkout, present only where it was checked out next to this build
REF = _reference_dir()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs an sm_103 GPU (run with -m gpu)")


@pytest.fixture(scope="session")
def oracle():
    import pyoracle

    pyoracle.build()
    pyoracle.lib()
    return pyoracle


@pytest.fixture(scope="session")
def enginelib():
    from gwgb300 import _lib

    return _lib.load(build_if_missing=True)


@pytest.fixture(scope="session")
def GW(enginelib):
    import GreensteinWinslow

    return GreensteinWinslow


@pytest.fixture(scope="session")
def ref_src(GW):
    if not os.path.isdir(os.path.join(REF, "src")):
        pytest.skip("reference Python layer not present")
    build = types.ModuleType("build")
    build.GreensteinWinslow = GW
    saved = {k: sys.modules.get(k) for k in ("build", "build.GreensteinWinslow", "h5py")}
    sys.modules["build"] = build
    sys.modules["build.GreensteinWinslow"] = GW
    h5 = types.ModuleType("h5py")
    h5.File = object
    sys.modules["h5py"] = h5
    sys.path.insert(0, REF)
    try:
        src = importlib.import_module("src")
        yield src
    finally:
        sys.path.remove(REF)
        for k, v in saved.items():
            if v is None:
                sys.modules.pop(k, None)
            else:
                sys.modules[k] = v
