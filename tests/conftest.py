import importlib.util
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "dendro-5.01_gb300")
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def load_dgb():
    spec = importlib.util.spec_from_file_location("dgb", os.path.join(PKG, "dgb.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="session")
def dgb():
    mod = load_dgb()
    if not os.path.exists(mod.LIB_PATH):
        sys.path.insert(0, PKG)
        import build  # noqa: E402
        build.build()
    return mod


@pytest.fixture(scope="session")
def oracle():
    import oracle_py
    oracle_py.build_oracle()
    return oracle_py.Oracle()


@pytest.fixture(scope="session")
def reference():
    import oracle_py
    if not os.path.isdir(oracle_py.REF_ROOT) and not os.path.exists(oracle_py.REF_SO):
        pytest.skip("reference tree not present on this machine")
    try:
        oracle_py.build_ref()
        return oracle_py.Reference()
    except Exception as e:  # pragma: no cover
        pytest.skip(f"reference build unavailable: {e}")


@pytest.fixture(scope="session")
def gpu(dgb):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    dgb.init(0)
    return torch
