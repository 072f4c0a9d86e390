"""GPU tests of the precision form (qh_pmatrix_*: tcgen05 f16 digit planes x
hi/mid/lo f16 limbs, FP32 accumulation in tensor memory, FP64 scales and
sums) against the plain FP64 form and the oracle.

Tolerances (stated):
* every matrix: ||y_pf - y_ref|| / ||y_ref|| <= 1e-5 (FP32-level
  accumulation; y_ref the oracle, i.e. the reference's matmul);
* the acceptance gate of the chosen form, per right-hand-side column:
  max |y_pf - y_plain| <= 0.01 * reconstruction_bound * ||x||_1.  The
  precision form is chosen per matrix by a calibration (choose_form); where it
  is chosen, the gate must hold on fresh right-hand sides, and where it is not,
  form="auto" must return the plain result bit for bit.
"""

import numpy as np
import pytest

from conftest import GOLDEN_CASES, golden, rel_err
from oracle import oracle as O
from qhmat_gb300 import HMatrix, PrecisionHMatrix, precision_gate

pytestmark = pytest.mark.gpu
REL = 1e-5


def _check(data, x):
    h = HMatrix.from_bytes(data, precision=True)
    y_pf = h.matmul(x, form="precision")
    y_plain = h.matmul(x)
    ref = O.OracleMatrix(data).matmul(x)
    assert rel_err(y_pf, ref) <= REL
    gate = precision_gate(y_pf, y_plain, x, h.reconstruction_bound)
    if h.form_choice["form"] == "precision":
        assert gate["passes"], (gate, h.form_choice)
        if np.ndim(x) == 2 and x.shape[1] >= 2:
            assert np.array_equal(h.matmul(x, form="auto"), y_pf)
    else:
        assert np.array_equal(h.matmul(x, form="auto"), y_plain)
    return y_pf, h


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_precision_form_against_plain_and_reference(cuda_device, name):
    data, g = golden(name)
    y_pf, h = _check(data, g["x"])
    assert rel_err(y_pf, g["y"]) <= REL
    x = np.random.default_rng(5).standard_normal((h.order, 64))
    _check(data, x)


@pytest.mark.parametrize("p", [1, 7, 16, 64, 100])
def test_precision_form_rhs_counts(cuda_device, p):
    """1 .. 64 right-hand sides in one pass, 100 in two passes (64 + 36)."""
    data, _ = golden("cfg1")
    x = np.random.default_rng(p).standard_normal((2048, p))
    y_pf, h = _check(data, x)
    if p == 100:
        # a column of the second pass agrees with its own one-column apply
        # (exponents are per column; only the MMA's N differs)
        y1 = h.matmul(np.ascontiguousarray(x[:, 70]), form="precision")
        assert rel_err(y1, y_pf[:, 70]) <= 1e-12


def test_precision_form_is_deterministic_and_column_independent(cuda_device):
    import torch

    data, _ = golden("ragged300")
    pm = PrecisionHMatrix.from_bytes(data)
    x = torch.from_numpy(np.random.default_rng(2).standard_normal((300, 24))).cuda()
    y1 = pm.matmul(x)
    y2 = pm.matmul(x)
    assert torch.equal(y1, y2)
    y5 = pm.matmul(x[:, 5].contiguous())
    assert rel_err(y5.cpu().numpy(), y1[:, 5].cpu().numpy()) <= 1e-12


def test_host_buffers_match_device_buffers(cuda_device):
    """qh_pmatmul_host (NumPy buffers: read and written in place by the
    kernels on a device that walks the host page tables, else staged through
    pinned memory) gives the tensor path's y bit for bit; an in-place call
    (x and y the same buffer) takes the staged path and agrees as well."""
    import ctypes as C

    import torch

    from qhmat_gb300 import _lib

    data, _ = golden("ragged300")
    pm = PrecisionHMatrix.from_bytes(data)
    x = np.random.default_rng(8).standard_normal((300, 70))
    y_dev = pm.matmul(torch.from_numpy(x).cuda()).cpu().numpy()
    y_host = pm.matmul(x)
    assert np.array_equal(y_host, y_dev)
    buf = x.copy()
    lib = _lib.load_library()
    _lib.raise_for(lib.qh_pmatmul_host(pm._h, buf.ctypes.data, buf.ctypes.data, C.c_size_t(70)))
    assert np.array_equal(buf, y_dev)
    assert pm.host_direct in (True, False)


def test_one_chunk_segments_are_closer_to_the_plain_form(cuda_device):
    """Accumulation segments of one K chunk (the setting calibration falls
    back to for tight tolerances) are deterministic and no farther from the
    plain form than the default two-chunk segments, in norm and in the gate's
    worst-column ratio (this fixture's tolerance is tighter than either
    setting meets); other settings are rejected."""
    data, _ = golden("ragged300")
    h = HMatrix.from_bytes(data)
    pm = PrecisionHMatrix.from_bytes(data)
    x = np.random.default_rng(21).standard_normal((300, 40))
    y_plain = h.matmul(x)
    assert pm.segment_chunks == 2
    y2 = pm.matmul(x)
    pm.segment_chunks = 1
    y1 = pm.matmul(x)
    assert np.array_equal(y1, pm.matmul(x))
    assert rel_err(y1, y_plain) <= max(rel_err(y2, y_plain), 1e-9) * 1.5
    r1 = precision_gate(y1, y_plain, x, h.reconstruction_bound)["worst_ratio"]
    r2 = precision_gate(y2, y_plain, x, h.reconstruction_bound)["worst_ratio"]
    assert r1 <= r2 * 1.5
    with pytest.raises(ValueError):
        pm.segment_chunks = 3
    assert pm.segment_chunks == 1


def test_precision_form_large_blocks_p64(cuda_device):
    """1-D n = 4096, -log(r + 1e-3), tolerance 1e-6: blocks up to 1024 columns,
    64 right-hand sides in one pass."""
    from qhmat_gb300 import construct

    rng = np.random.default_rng(11)
    pts = rng.random((4096, 1))
    img = construct.from_kernel(pts, "log", tolerance=1e-6, leaf_size=64, workers=8)
    data = construct.to_qhmat_bytes(img, checksum=O.fnv1a64)
    x = rng.standard_normal((4096, 64))
    _check(data, x)


def test_precision_form_nonfinite(cuda_device):
    data, g = golden("cfg1")
    pm = PrecisionHMatrix.from_bytes(data)
    x = g["x"].copy()
    x[3, 1] = np.nan
    with pytest.raises(ValueError, match="nonfinite right-hand side"):
        pm.matmul(x)
