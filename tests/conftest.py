import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "golden_*.npz")))


def _reference_root():
    import oracle

    return oracle.reference_root()


# where the reference's sources lie (the oracle's build recipe knows); the
# tests that read them skip when they are absent
REFERENCE = _reference_root()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def orc():
    import oracle

    return oracle.Oracle()


@pytest.fixture(scope="session")
def ref():
    import oracle

    if not os.path.isdir(os.path.join(REFERENCE, "v25")):
        pytest.skip("reference sources not present")
    if not os.path.exists(oracle.REF_SO):
        oracle.build_ref()
    return oracle.Ref()


@pytest.fixture(scope="session")
def ref_serial():
    """The reference built without OpenMP: its loops' dynamic schedule takes
    a chunk of 0 below 16 particles per thread and never ends there."""
    import oracle

    if not os.path.isdir(os.path.join(REFERENCE, "v25")):
        pytest.skip("reference sources not present")
    if not os.path.exists(oracle.REF_SERIAL_SO):
        oracle.build_ref()
    return oracle.Ref(oracle.REF_SERIAL_SO)


def rms_rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.sqrt(np.mean(b ** 2))
    return float(np.sqrt(np.mean((a - b) ** 2)) / den) if den > 0 else float(np.abs(a).max())


def load_golden(path):
    return dict(np.load(path))
