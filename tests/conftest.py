import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN_CASES = ["tiny2", "kernel12", "zero_rank", "packed8", "cuda10", "ragged300", "cfg1"] + [
    f"orth17_b{b}" for b in (2, 4, 8, 12, 16, 24, 32)]


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


def golden(name: str):
    """(qhmat bytes, npz dict) of a fixture produced by tests/golden/make_golden.py."""
    data = (GOLDEN / f"{name}.qhmat").read_bytes()
    arrs = dict(np.load(GOLDEN / f"{name}.npz"))
    return data, arrs


def rel_err(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb else 1.0))


@pytest.fixture(scope="session")
def cuda_device():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return 0
