"""The C ABI library: loads, exports what include/qhmat_gb300.h declares, and
reports host-side errors with the reference's types and messages (CPU-only)."""

import ctypes as C
import re

import numpy as np
import pytest

from conftest import ROOT, golden
from qhmat_gb300 import HMatrix, _lib


def _declared_symbols():
    text = (ROOT / "include" / "qhmat_gb300.h").read_text()
    return sorted(set(re.findall(r"QH_API\s+[\w\s\*]+?\b(qh_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = _lib.load_library()
    names = _declared_symbols()
    assert len(names) >= 11
    for name in names:
        assert hasattr(lib, name), name
    assert lib.qh_cuda_built() == 1


def test_library_is_the_in_tree_build():
    assert _lib.LIB_PATH.parent == ROOT / "qhmat_gb300"
    assert _lib.LIB_PATH.exists()


@pytest.mark.parametrize("mutate,exc,match", [
    (lambda d: d[:-5], RuntimeError, "truncated|trailing"),
    (lambda d: d[:-9] + bytes([d[-9] ^ 1]) + d[-8:], RuntimeError, "checksum mismatch"),
    (lambda d: b"QHMAT002" + d[8:], RuntimeError, "invalid qhmat file magic"),
    (lambda d: d[:8] + (2).to_bytes(8, "little") + d[16:], RuntimeError, "unsupported qhmat file version"),
    (lambda d: d[:16] + (0).to_bytes(8, "little") + d[24:], RuntimeError, "invalid qhmat file dimensions"),
    (lambda d: d[:10], RuntimeError, "truncated qhmat file"),
])
def test_corrupt_images_raise_reference_errors(mutate, exc, match):
    data, _ = golden("packed8")
    with pytest.raises(exc, match=match):
        HMatrix.from_bytes(mutate(data))


def _rehash(body: bytes) -> bytes:
    h = 14695981039346656037
    for b in body:
        h = ((h ^ b) * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return body + h.to_bytes(8, "little")


def test_permutation_and_partition_checks():
    data, _ = golden("tiny2")
    body = bytearray(data[:-8])
    # permutation [0, 1] -> [0, 0]
    body[40:48] = (0).to_bytes(8, "little")
    with pytest.raises(ValueError, match="permutation is not a bijection"):
        HMatrix.from_bytes(_rehash(bytes(body)))
    # shrink the first block's row1/col1 so the partition has a gap
    body = bytearray(data[:-8])
    off = 8 + 24 + 16
    assert int.from_bytes(body[off + 8:off + 16], "little") == 1
    # the flag bytes of block 0 sit after its rectangle; mark it non-dense -> rectangle check
    body[off + 33] = 0
    with pytest.raises((ValueError, RuntimeError)):
        HMatrix.from_bytes(_rehash(bytes(body)))


def test_no_device_error_without_gpu():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    data, _ = golden("cuda10")
    with pytest.raises(RuntimeError, match="no CUDA device is available|cudaGetDeviceCount"):
        HMatrix.from_bytes(data)


def test_from_arrays_validation_without_gpu():
    # a partition gap is rejected before any device work
    with pytest.raises(ValueError, match="partition"):
        HMatrix.from_arrays(2, [0, 1], [(0, 1, 0, 1, 0, 0, 0, 1)], np.array([2.0]),
                            np.zeros(1, np.uint32), np.zeros(1, np.uint32), [], [], [], [], [])
    with pytest.raises(ValueError, match="bijection"):
        HMatrix.from_arrays(2, [1, 1], [(0, 1, 0, 1, 0, 0, 0, 1), (1, 2, 1, 2, 0, 0, 1, 1)],
                            np.array([2.0, 3.0]), np.zeros(1, np.uint32), np.zeros(1, np.uint32),
                            [], [], [], [], [])
