import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "goofy_golden.npz")

# Tests run with the compiled default tiles: no tuned tiles from a per-user
# cache file of an earlier run.  The tile-cache tests give their own paths.
os.environ.setdefault("GOOFY_TILE_CACHE", "")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built():
    """Build the library, the synthetic-workload generator and the oracle once."""
    from goofy_gb300 import build as lib_build
    from oracle import build as oracle_build

    oracle_build.build()
    lib_build.build()
    return True


@pytest.fixture(scope="session")
def golden():
    return dict(np.load(GOLDEN))


@pytest.fixture(scope="session")
def oracle_lib(built):
    import oracle

    return oracle.load()


@pytest.fixture(scope="session")
def cuda(built):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)
    import goofy_gb300 as g

    assert g.init(0) == g.OK, g.last_error()
    return torch
