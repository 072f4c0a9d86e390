"""Generate the golden fixtures in tests/golden/ with the reference itself.

Run in a container that has the reference sources (default /root/reference,
override with QHMAT_REFERENCE):

    python tests/golden/make_golden.py

For every case the reference's own Python API builds the matrix (the same
inputs as the reference's tests/test_core.py and tests/test_cuda.py, plus the
CPU-runnable plain configuration at n=2048), saves it with ``HMatrix.save``
(QHMAT001), and applies its CPU ``matmul`` to seeded right-hand sides.  Each
case writes ``<name>.qhmat`` and ``<name>.npz`` with:

    x      the right-hand side (row-major, source order)
    y      the reference's ``matmul(x)``
    bound  the reference's ``reconstruction_bound``
    dense  the reference's ``to_dense()`` (small cases only)

The fixtures pin the CPU oracle (oracle/qhmat_oracle.c) and are the parity
targets of the GPU tests; the reference is not needed to run the tests.
"""

from __future__ import annotations

import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

from oracle.build_ref import import_reference_qhmat  # noqa: E402


def _save(q, name, matrix, x, dense: bool):
    path = HERE / f"{name}.qhmat"
    if path.exists():
        path.unlink()
    matrix.save(str(path))
    native = matrix if isinstance(matrix, q.NativeHMatrix) else matrix._native
    y = native.matmul(np.asarray(x, dtype=np.float64))
    extra = {"dense": native.reconstruct()} if dense else {}
    np.savez(HERE / f"{name}.npz", x=np.asarray(x, np.float64), y=y,
             bound=np.float64(native.reconstruction_bound), **extra)
    print(f"{name}: order={native.order} bytes={path.stat().st_size}")


def main() -> None:
    q = import_reference_qhmat()

    # tests/test_core.py:44-60 -- exact 2x2 apply
    m = q.NativeHMatrix(2, [0, 1])
    m.add_dense(q.Rectangle(0, 1, 0, 1), np.array([[2.0]]))
    m.add_dense(q.Rectangle(1, 2, 1, 2), np.array([[3.0]]))
    for row, col in [(0, 1), (1, 0)]:
        m.add_low_rank(q.Rectangle(row, row + 1, col, col + 1), np.ones((1, 1)),
                       np.array([1.0]), np.ones((1, 1)), [8], 3, 0.0)
    m.finalize()
    _save(q, "tiny2", m, np.eye(2), dense=True)

    # tests/test_core.py:70-83 -- kernel 1/(r+0.4), n=12, leaf 3
    pts = np.linspace(0, 1, 12)[:, None]
    src = 1.0 / (np.abs(pts - pts.T) + 0.4)
    h = q.HMatrix.from_dense(src, pts, tolerance=0.25, leaf_size=3, bit_widths=(4, 8, 16, 32))
    _save(q, "kernel12", h, np.eye(12), dense=True)

    # tests/test_core.py:154-167 -- permutation [1, 0] and rank-0 off-diagonal blocks
    rects = [q.Rectangle(0, 1, 0, 1), q.Rectangle(0, 1, 1, 2), q.Rectangle(1, 2, 0, 1),
             q.Rectangle(1, 2, 1, 2)]
    h = q.HMatrix.from_partition(np.diag([2.0, 3.0]), np.array([1, 0], dtype=np.int64), rects,
                                 tolerance=0.1)
    _save(q, "zero_rank", h, np.array([[1.0, -2.0], [0.5, 4.0]]), dense=True)

    # tests/test_core.py:170-192 -- random orthogonal factors at every width
    for bit in (2, 4, 8, 12, 16, 24, 32):
        rng = np.random.default_rng(200 + bit)
        u, _ = np.linalg.qr(rng.normal(size=(9, 3)))
        v, _ = np.linalg.qr(rng.normal(size=(8, 3)))
        sigma = np.array([3.0, 1.0, 0.2])
        native = q.NativeHMatrix(17, list(range(17)))
        native.add_dense(q.Rectangle(0, 9, 0, 9), np.eye(9))
        native.add_dense(q.Rectangle(9, 17, 9, 17), np.eye(8))
        native.add_low_rank(q.Rectangle(0, 9, 9, 17), u, sigma, v, [bit] * 3, 1, 0.0)
        native.add_low_rank(q.Rectangle(9, 17, 0, 9), v, sigma, u, [bit] * 3, 1, 0.0)
        native.finalize()
        _save(q, f"orth17_b{bit}", native, rng.normal(size=(17, 4)), dense=True)

    # tests/test_core.py:205-232 -- n=8, leaf 2
    pts = np.linspace(0, 1, 8)[:, None]
    src = 1.0 / (0.4 + np.abs(pts - pts.T))
    h = q.HMatrix.from_dense(src, pts, tolerance=0.25, leaf_size=2, bit_widths=(4, 8, 16, 32))
    _save(q, "packed8", h, np.eye(8), dense=True)

    # tests/test_cuda.py:8-23 -- n=10, leaf 2, RHS seed 11, shape 10x3
    pts = np.linspace(0.0, 1.0, 10)[:, None]
    src = 1.0 / (0.4 + np.abs(pts - pts.T))
    h = q.HMatrix.from_dense(src, pts, tolerance=0.25, leaf_size=2, bit_widths=(4, 8, 16, 32))
    _save(q, "cuda10", h, np.random.default_rng(11).normal(size=(10, 3)), dense=True)

    # Mixed widths at every menu entry, 2-D points, ragged leaves (n=300, leaf 7)
    rng = np.random.default_rng(5)
    pts = rng.random((300, 2))
    r = np.sqrt(((pts[:, None, :] - pts[None, :, :]) ** 2).sum(-1))
    src = -np.log(r + 1e-3)
    h = q.HMatrix.from_dense(src, pts, tolerance=1e-6, leaf_size=7,
                             bit_widths=(2, 3, 4, 5, 8, 11, 12, 16, 17, 24, 31, 32))
    _save(q, "ragged300", h, rng.standard_normal((300, 3)), dense=False)

    # Plain configuration 1: n=2048 1-D, 1/(r+0.4), leaf 32, tol 1e-6, X 2048x4 seed 0
    pts = np.linspace(0, 1, 2048)[:, None]
    src = 1.0 / (np.abs(pts - pts.T) + 0.4)
    h = q.HMatrix.from_dense(src, pts, tolerance=1e-6, leaf_size=32,
                             bit_widths=(4, 8, 12, 16, 24, 32))
    _save(q, "cfg1", h, np.random.default_rng(0).standard_normal((2048, 4)), dense=False)


if __name__ == "__main__":
    main()
