"""CPU check of the precision form's resident layout: tests/pf_layout_check.cpp
(built here with g++ from the library's layout.cpp and pf_layout.cpp) walks
the work lists the tcgen05 kernels walk, in FP64 with the digit planes
recombined into codes and the swizzled dense limb tiles un-swizzled, and must
reproduce the oracle's y (the reference's matmul restated) up to the
~33-bit representation of the dense blocks by three f16 limbs.
No GPU."""

import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from conftest import GOLDEN_CASES, golden, rel_err
from oracle import oracle as O

ROOT = Path(__file__).resolve().parents[1]
CSRC = ROOT / "qhmat_gb300" / "csrc"


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    exe = tmp_path_factory.mktemp("pf") / "pf_layout_check"
    subprocess.run(["g++", "-O2", "-std=c++17", f"-I{CSRC}", "-o", str(exe),
                    str(ROOT / "tests" / "pf_layout_check.cpp"), str(CSRC / "layout.cpp"),
                    str(CSRC / "pf_layout.cpp")], check=True, capture_output=True, text=True)
    return exe


def _run(checker, tmp_path, data: bytes, x: np.ndarray, grid: int):
    f = tmp_path / "m.qhmat"
    f.write_bytes(data)
    fx, fy = tmp_path / "x.bin", tmp_path / "y.bin"
    np.ascontiguousarray(x, np.float64).tofile(fx)
    r = subprocess.run([str(checker), str(f), str(fx), str(fy), str(grid)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("OK"), r.stdout
    return np.fromfile(fy, np.float64)


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_pf_layout_reproduces_oracle(checker, tmp_path, name):
    data, g = golden(name)
    m = O.OracleMatrix(data)
    x = np.random.default_rng(3).standard_normal(m.order)
    for grid in (1, 5):
        y = _run(checker, tmp_path, data, x, grid)
        assert rel_err(y, m.matmul(x)) <= 1e-9  # dense blocks as three f16 limbs: ~33 bits


def test_pf_layout_large_blocks(checker, tmp_path):
    """1-D n = 4096: blocks up to 1024 columns (column items of 16 chunks,
    128-row tiles met by wide blocks), on the 152-block schedule."""
    from qhmat_gb300 import construct

    rng = np.random.default_rng(11)
    pts = rng.random((4096, 1))
    img = construct.from_kernel(pts, "log", tolerance=1e-6, leaf_size=64, workers=4)
    data = construct.to_qhmat_bytes(img, checksum=O.fnv1a64)
    m = O.OracleMatrix(data)
    x = rng.standard_normal(4096)
    y = _run(checker, tmp_path, data, x, 152)
    assert rel_err(y, m.matmul(x)) <= 1e-9
