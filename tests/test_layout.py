"""CPU checks of the resident layout the kernels read: every code decoded
back from the stored digit planes (column and row side) equals the reference's
decode of the QHMAT001 file, every B row slot is written by exactly one
column task of its component, dense slices cover the dense blocks once, and
the row pipeline's uniform-step marks agree with the k-pair infos.  Built from
the library's own layout.cpp with g++ (tests/layout_check.cpp); no GPU."""

import shutil
import subprocess
from pathlib import Path

import pytest

from conftest import GOLDEN_CASES

ROOT = Path(__file__).resolve().parents[1]
CSRC = ROOT / "qhmat_gb300" / "csrc"


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    exe = tmp_path_factory.mktemp("layout") / "layout_check"
    subprocess.run(["g++", "-O2", "-std=c++17", f"-I{CSRC}", "-o", str(exe),
                    str(ROOT / "tests" / "layout_check.cpp"), str(CSRC / "layout.cpp")],
                   check=True, capture_output=True, text=True)
    return exe


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_layout_round_trip(checker, name):
    r = subprocess.run([str(checker), str(ROOT / "tests" / "golden" / f"{name}.qhmat")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("OK")


@pytest.mark.parametrize("name", ["ragged300", "cfg1", "orth17_b12"])
def test_layout_round_trip_with_split_tasks(checker, name):
    """The same checks with every column task longer than one chunk split into
    one-chunk parts (QHMAT_GB300_PART_CHUNKS=1), the layout the split-task
    path of the column kernel reads."""
    import os

    env = dict(os.environ, QHMAT_GB300_PART_CHUNKS="1")
    r = subprocess.run([str(checker), str(ROOT / "tests" / "golden" / f"{name}.qhmat")],
                       capture_output=True, text=True, env=env)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("OK")
