import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_DIR = os.path.join(ROOT, "chaos-ultra_gb300")
for p in (PKG_DIR, ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300 box)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import build_oracle
    from oracle.oracle import Oracle

    build_oracle.build_oracle()
    return Oracle()


@pytest.fixture(scope="session")
def reference():
    """The reference's own computeFractal built for this host, or skip."""
    from oracle import build_oracle
    from oracle.oracle import REF_LIB, Reference

    try:
        build_oracle.build_reference()
    except RuntimeError as e:
        pytest.skip(f"reference build unavailable: {str(e).splitlines()[0]}")
    if not os.path.exists(REF_LIB):
        pytest.skip("reference sources not present on this machine")
    return Reference()


@pytest.fixture(scope="session")
def native():
    """libchaos_gb300.so, built in-tree if needed."""
    import chaos_gb300

    if not os.path.exists(chaos_gb300.LIB_PATH):
        import importlib.util

        spec = importlib.util.spec_from_file_location("bn", os.path.join(PKG_DIR, "build_native.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build()
    return chaos_gb300.lib()


@pytest.fixture(scope="session")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)
    torch.zeros(1, device="cuda:0")  # create the primary context
    return torch
