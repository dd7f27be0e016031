import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "barnes-hut_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the CUDA kernels)")


def golden_cases():
    return sorted(f[4:-4] for f in os.listdir(GOLDEN) if f.startswith("ref_") and f.endswith(".npz"))


def ensure_library():
    """Compile libbh_gb300.so in-tree if this checkout has not built it yet (nvcc cross-compiles
    for sm_103a without a GPU), so the loading and symbol tests run on a fresh checkout."""
    from barneshut.gb300 import native

    if not os.path.exists(native.LIB_PATH):
        import importlib.util

        spec = importlib.util.spec_from_file_location("bh_build", os.path.join(PKG, "build.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build()
    return native


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle

    oracle.build()
    return oracle
