import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the library and the oracle once per session (incremental)."""
    import __graft_entry__
    __graft_entry__.build()


def rel_force_err(f, ref):
    """max_i |dF_i| / max(|F_ref,i|, 1e-3 F_rms)."""
    fr = np.linalg.norm(ref, axis=1)
    floor = 1e-3 * np.sqrt(np.mean(fr ** 2))
    return float(np.max(np.linalg.norm(f - ref, axis=1) / np.maximum(fr, floor)))


def rms_rel_err(f, ref):
    return float(np.sqrt(np.sum((f - ref) ** 2) / np.sum(ref ** 2)))


@pytest.fixture
def gpu():
    import opencafemol_gb300 as ocm
    if ocm.device_count() < 1:
        pytest.fail("a GPU test ran without a CUDA device")
    return ocm
