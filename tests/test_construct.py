"""The restated construction (qhmat_gb300/construct.py) against the reference.

The bench builds its workload on the GPU host with construct.py because the
reference cannot be installed there; these tests pin that restatement to the
reference's own output: the QHMAT001 images of the golden fixtures were
written by the reference's ``HMatrix.from_dense(...).save`` (see
tests/golden/make_golden.py), and the restated construction must reproduce
them byte for byte on the same NumPy build.  ``pack`` is also checked against
the oracle's restatement of ``HMatrix::pack`` (src/qhmat/core.cpp:235-267).
"""

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import oracle as O
from qhmat_gb300 import construct as K


def _golden_bytes(name):
    return (GOLDEN / f"{name}.qhmat").read_bytes()


def test_cfg1_image_is_byte_identical():
    """n=2048 points on [0, 1], 1/(r+0.4), leaf 32, tolerance 1e-6."""
    pts = np.linspace(0, 1, 2048)[:, None]
    img = K.from_kernel(pts, "inverse", tolerance=1e-6, leaf_size=32, workers=4)
    assert K.to_qhmat_bytes(img) == _golden_bytes("cfg1")


def test_ragged300_image_is_byte_identical():
    """2-D points, -log(r+1e-3), leaf 7, twelve widths (every menu entry used)."""
    rng = np.random.default_rng(5)
    pts = rng.random((300, 2))
    img = K.from_kernel(pts, "log", tolerance=1e-6, leaf_size=7,
                        bit_widths=(2, 3, 4, 5, 8, 11, 12, 16, 17, 24, 31, 32), workers=1)
    assert K.to_qhmat_bytes(img) == _golden_bytes("ragged300")


@pytest.mark.parametrize("bits", [2, 3, 7, 8, 13, 16, 24, 31, 32])
def test_pack_matches_oracle(bits):
    rng = np.random.default_rng(bits)
    m = rng.normal(size=(37, 5)) * np.logspace(0, -3, 5)
    widths = [bits] * 5
    words, scales = K.pack(m, widths)
    ow, oo, os_ = O.pack(m, widths)
    np.testing.assert_array_equal(np.asarray(words, dtype=np.uint32), ow)
    np.testing.assert_array_equal(np.asarray(scales, dtype=np.float64), os_)


def test_invalid_arguments_raise():
    pts = np.linspace(0, 1, 16)[:, None]
    with pytest.raises(ValueError):
        K.from_kernel(pts, "inverse", tolerance=0.0)
    with pytest.raises(ValueError):
        K.from_kernel(pts, "inverse", tolerance=1e-6, bit_widths=(1, 8))
    with pytest.raises(ValueError):
        K.from_kernel(pts, "nope", tolerance=1e-6)


def test_randomized_svd_path_builds_a_valid_matrix():
    """The fast construction path: every block passes the reference's
    residual and allocation checks, the matrix applies like the dense kernel
    matrix within its bound, and it is deterministic."""
    import numpy as np

    from oracle import oracle as O
    from qhmat_gb300 import construct

    rng = np.random.default_rng(3)
    pts = rng.random((2048, 1))
    img = construct.from_kernel(pts, "log", tolerance=1e-6, leaf_size=32, workers=1, svd="randomized")
    data = construct.to_qhmat_bytes(img, checksum=O.fnv1a64)
    again = construct.to_qhmat_bytes(construct.from_kernel(pts, "log", tolerance=1e-6, leaf_size=32, workers=1,
                                                           svd="randomized"), checksum=O.fnv1a64)
    assert data == again
    m = O.OracleMatrix(data)
    x = rng.standard_normal(2048)
    a = construct.kernel_matrix(pts, "log")
    err = np.max(np.abs(m.matmul(x) - a @ x))
    assert err <= m.reconstruction_bound * np.sum(np.abs(x))
    assert max(b.rank for b in img.blocks if b.dense is None) <= 96
