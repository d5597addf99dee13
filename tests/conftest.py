import json
import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
GOLDEN = ROOT / "tests" / "golden"
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a); parity tests through the C ABI")
    config.addinivalue_line("markers", "slow: longer CPU test")


@pytest.fixture(scope="session")
def built():
    """Build libecsgpu / libecshost and the oracle once per session."""
    from ecsprt_gb300 import build as b
    from oracle import oracle as orc

    b.build()
    orc.build()
    return True


def load_golden(name):
    d = dict(np.load(GOLDEN / f"{name}.npz", allow_pickle=False))
    if "params" in d:
        d["params"] = json.loads(str(d["params"]))
    if "opts" in d:
        d["opts"] = str(d["opts"])
    return d


@pytest.fixture(scope="session")
def golden():
    return {n: load_golden(n) for n in ("c1", "edge", "fb", "rng")}


def have_gpu():
    """True when the CUDA runtime reports at least one device."""
    import ctypes

    for name in ("libcudart.so.13", "/usr/local/cuda/lib64/libcudart.so.13", "libcudart.so"):
        try:
            rt = ctypes.CDLL(name)
        except OSError:
            continue
        n = ctypes.c_int(0)
        return rt.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0
    return False


def pytest_collection_modifyitems(config, items):
    if os.environ.get("ECSPRT_FORCE_GPU"):
        return
    if not have_gpu():
        skip = pytest.mark.skip(reason="no CUDA device")
        for it in items:
            if "gpu" in it.keywords:
                it.add_marker(skip)
