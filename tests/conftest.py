import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity tests through the C-ABI")


def pytest_sessionstart(session):
    # build the library and the CPU oracle if this checkout has not built them yet
    from openol_gb300 import build as B
    if not os.path.exists(B.LIB):
        B.build()
    import oracle
    if not os.path.exists(os.path.join(oracle.HERE, "libolcpu.so")):
        oracle.build()


def pytest_collection_modifyitems(config, items):
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    return np.load(os.path.join(ROOT, "tests", "golden", "ref_golden.npz"))


@pytest.fixture(scope="session")
def golden_dir():
    import pathlib
    return pathlib.Path(ROOT) / "tests" / "golden"


def rel_l2(a, b):
    import numpy as np
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
