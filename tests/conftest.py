"""Shared test set-up: the `gpu` marker, import paths for the package (whose folder
name, quicklabpiv-ng_gb300, is not a Python identifier) and for the CPU oracle."""
import importlib.util
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"
sys.path.insert(0, str(ROOT / "oracle"))


def load_package():
    name = "quicklabpiv_ng_gb300"
    if name in sys.modules:
        return sys.modules[name]
    pkg_dir = ROOT / "quicklabpiv-ng_gb300"
    spec = importlib.util.spec_from_file_location(name, pkg_dir / "__init__.py",
                                                  submodule_search_locations=[str(pkg_dir)])
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    import oracle as orc
    orc.lib()
    return orc


@pytest.fixture(scope="session")
def rankine_pair():
    d = np.load(GOLDEN / "rankine_pair.npz")
    return d["a"], d["b"]
