"""Shared test setup: the `gpu` marker, the oracle and the package loader."""
import importlib.util
import json
import pathlib
import sys

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = json.loads((ROOT / "tests" / "golden" / "cfrg_bls12381_sha256.json").read_text())


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")


def load_package():
    """Import cubbs-cred_gb300/ (hyphenated directory) as module cubbs_gb300."""
    if "cubbs_gb300" in sys.modules:
        return sys.modules["cubbs_gb300"]
    pkg = ROOT / "cubbs-cred_gb300"
    spec = importlib.util.spec_from_file_location("cubbs_gb300", pkg / "__init__.py",
                                                  submodule_search_locations=[str(pkg)])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["cubbs_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="session")
def golden():
    return GOLDEN


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle_ctypes
    oracle_ctypes.lib()
    return oracle_ctypes


@pytest.fixture(scope="session")
def gpu():
    """The CUDA library (built in-tree if needed)."""
    mod = load_package()
    mod.build()
    kind, hw = mod.backend_info()
    assert kind == mod.BACKEND_KIND_CUDA and hw == 1, "CUDA backend unavailable"
    return mod
