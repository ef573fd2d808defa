import os
import sys
import zlib

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "swarm-crowd-simulation_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if _has_gpu():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


@pytest.fixture(scope="session")
def built():
    """The CUDA library and the oracle, built in-tree (a no-op when up to date)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("swarm_pkg_build", os.path.join(PKG, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build()
    from oracle import oracle as O
    O.build()
    return True


@pytest.fixture(scope="session")
def stadium_sdf():
    raw = zlib.decompress(open(os.path.join(GOLDEN, "stadium_sdf.zlib"), "rb").read())
    return np.frombuffer(raw, dtype=np.float32).copy()


@pytest.fixture(scope="session")
def terrace_golden():
    return dict(np.load(os.path.join(GOLDEN, "terrace_ref.npz")))
