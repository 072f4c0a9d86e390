"""GPU parity of the resident matvec against the reference (via its golden
fixtures) and the CPU oracle.  Every call goes through the C ABI
(libqhmat_gb300.so) -- there is no other compute path.

Tolerance (stated by the build target): ||y - y_ref|| / ||y_ref|| <= 1e-13,
with y_ref the reference's CPU HMatrix::matmul on identical inputs; code
unpacking is compared bit-for-bit.
"""

import numpy as np
import pytest

from conftest import GOLDEN_CASES, golden, rel_err
from oracle import oracle as O
from qhmat_gb300 import HMatrix, NativeHMatrix

pytestmark = pytest.mark.gpu
TOL = 1e-13


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_matmul_matches_reference(cuda_device, name):
    data, g = golden(name)
    h = HMatrix.from_bytes(data)
    y = h.matmul(g["x"], device="cuda")
    assert y.shape == g["y"].shape
    assert rel_err(y, g["y"]) <= TOL
    # column-wise too: every right-hand side on its own
    x2 = g["x"] if g["x"].ndim == 2 else g["x"][:, None]
    y2 = g["y"] if g["y"].ndim == 2 else g["y"][:, None]
    for p in range(x2.shape[1]):
        yp = h.matmul(np.ascontiguousarray(x2[:, p]))
        assert yp.shape == (h.order,)
        assert rel_err(yp, y2[:, p]) <= TOL
    assert h.reconstruction_bound == float(g["bound"])


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_codes_round_trip_bit_exact(cuda_device, name):
    """Codes decoded by the device routine == the reference decode, bit for bit."""
    data, _ = golden(name)
    h = HMatrix.from_bytes(data)
    m = O.OracleMatrix(data)
    for side in (0, 1):
        expect = [m.codes(b, side).ravel() for b in range(m.block_count)
                  if not m.block_info(b)["dense"]]
        expect = np.concatenate(expect) if expect else np.zeros(0, np.int32)
        got = h.debug_decode(side)
        assert got.dtype == np.int32 and np.array_equal(got, expect)


def test_tensor_path_matches_host_path_and_is_deterministic(cuda_device):
    import torch

    data, g = golden("cfg1")
    h = HMatrix.from_bytes(data)
    x = torch.from_numpy(g["x"]).cuda()
    y1 = h.matmul(x)
    y2 = h.matmul(x)
    assert y1.is_cuda and y1.dtype == torch.float64
    assert torch.equal(y1, y2), "two applies differ bitwise"
    assert np.array_equal(y1.cpu().numpy(), h.matmul(g["x"]))
    assert rel_err(y1.cpu().numpy(), g["y"]) <= TOL


def test_random_rhs_against_oracle(cuda_device):
    for name in ("ragged300", "cfg1"):
        data, _ = golden(name)
        h = HMatrix.from_bytes(data)
        m = O.OracleMatrix(data)
        rng = np.random.default_rng(99)
        for shape in [(m.order,), (m.order, 1), (m.order, 7)]:
            x = rng.standard_normal(shape)
            assert rel_err(h.matmul(x), m.matmul(x, threads=4)) <= TOL
        # graded magnitudes: entries spread over 2^-40 .. 2^40
        x = rng.standard_normal(m.order) * np.exp2(rng.integers(-40, 40, m.order))
        assert rel_err(h.matmul(x), m.matmul(x)) <= TOL
        # zeros and a single spike
        assert np.array_equal(h.matmul(np.zeros(m.order)), np.zeros(m.order))
        e = np.zeros(m.order)
        e[m.order // 3] = 1.0
        assert rel_err(h.matmul(e), m.matmul(e)) <= TOL


def test_errors_match_reference(cuda_device):
    data, g = golden("cuda10")
    h = HMatrix.from_bytes(data)
    x = g["x"].copy()
    x[2, 1] = np.inf
    with pytest.raises(ValueError, match="nonfinite right-hand side"):
        h.matmul(x)
    with pytest.raises(ValueError, match="wrong row count"):
        h.matmul(np.ones(11))
    with pytest.raises(ValueError, match="one- or two-dimensional"):
        h.matmul(np.ones((10, 2, 2)))
    with pytest.raises(ValueError, match="device must be"):
        h.matmul(g["x"], device="tpu")
    # still usable after an error
    assert rel_err(h.matmul(g["x"]), g["y"]) <= TOL
    n = NativeHMatrix.from_bytes(data)
    assert rel_err(n.matmul(g["x"], True), g["y"]) <= TOL


def test_from_arrays_matches_file_path(cuda_device):
    """The flat-array entry (the arrays matmul_cuda builds) gives the same result."""
    data, g = golden("ragged300")
    m = O.OracleMatrix(data)
    import struct

    blocks, dense, lw, rw, loff, roff, ls, rs, widths = [], [], [], [], [], [], [], [], []
    off = 8 + 24
    perm = np.frombuffer(data, np.uint64, m.order, off).astype(np.uintp)
    off += 8 * m.order
    dense_n = 0
    for b in range(m.block_count):
        info = m.block_info(b)
        rows, cols = info["row1"] - info["row0"], info["col1"] - info["col0"]
        off += 34
        if info["dense"]:
            blocks.append((info["row0"], info["row1"], info["col0"], info["col1"], 0, 0, dense_n, 1))
            dense.append(np.frombuffer(data, np.float64, rows * cols, off))
            dense_n += rows * cols
            off += 8 * rows * cols
            continue
        rank = info["rank"]
        off += 32
        w = np.frombuffer(data, np.uint8, rank, off).astype(np.intc)
        off += rank
        lsc = np.frombuffer(data, np.float64, rank, off)
        rsc = np.frombuffer(data, np.float64, rank, off + 8 * rank)
        off += 16 * rank
        blocks.append((info["row0"], info["row1"], info["col0"], info["col1"], rank, len(widths), 0, 0))
        lbase, rbase = sum(len(a) for a in lw), sum(len(a) for a in rw)
        lo = ro = 0
        for j in range(rank):
            loff.append(lbase + lo)
            roff.append(rbase + ro)
            lo += (rows * int(w[j]) + 31) // 32
            ro += (cols * int(w[j]) + 31) // 32
        lw.append(np.frombuffer(data, np.uint32, lo, off))
        rw.append(np.frombuffer(data, np.uint32, ro, off + 4 * lo))
        off += 4 * (lo + ro)
        widths.extend(w)
        ls.extend(lsc)
        rs.extend(rsc)
    h = HMatrix.from_arrays(m.order, perm, blocks, np.concatenate(dense), np.concatenate(lw),
                            np.concatenate(rw), loff, roff, ls, rs, widths)
    ref = HMatrix.from_bytes(data)
    assert np.array_equal(h.matmul(g["x"]), ref.matmul(g["x"]))


@pytest.mark.parametrize("name", [n for n in GOLDEN_CASES if n not in ("ragged300", "cfg1")])
def test_to_dense_bit_exact(cuda_device, name):
    """GPU reconstruct == the reference's HMatrix::reconstruct, bit for bit."""
    data, g = golden(name)
    h = HMatrix.from_bytes(data)
    dense = h.to_dense()
    assert dense.shape == (h.order, h.order)
    np.testing.assert_array_equal(dense, g["dense"])
    np.testing.assert_array_equal(NativeHMatrix.from_bytes(data).reconstruct(), g["dense"].reshape(-1))


def test_to_dense_matches_oracle_reconstruct(cuda_device):
    data, _ = golden("ragged300")
    h = HMatrix.from_bytes(data)
    np.testing.assert_array_equal(h.to_dense(), O.OracleMatrix(data).reconstruct())


def test_host_apply_in_place_matches(cuda_device):
    """qh_matmul_host with x and y in one buffer (which takes the pinned
    staging path even where the kernels can reach host memory directly)
    gives the same y, bit for bit, as the out-of-place call."""
    import ctypes as C

    from qhmat_gb300 import _lib

    data, g = golden("cfg1")
    h = HMatrix.from_bytes(data)
    x = np.ascontiguousarray(g["x"], dtype=np.float64)
    y = h.matmul(x, device="cuda")
    buf = x.copy()
    lib = _lib.load_library()
    rc = lib.qh_matmul_host(h._h, buf.ctypes.data_as(C.c_void_p), buf.ctypes.data_as(C.c_void_p), x.shape[1])
    assert rc == 0
    assert np.array_equal(buf, y)
    assert rel_err(buf, g["y"]) <= TOL


def test_many_rhs_columns_match_single_column_applies(cuda_device):
    """200 right-hand sides at n=2048 (more prep blocks than the device holds
    at once, so prep and limbs run as two launches instead of one cooperative
    launch): every column equals its own single-column apply bit for bit, and
    the reference's result within the tolerance."""
    data, g = golden("cfg1")
    h = HMatrix.from_bytes(data)
    m = O.OracleMatrix(data)
    x = np.random.default_rng(7).standard_normal((h.order, 200))
    y = h.matmul(x, device="cuda")
    for p in (0, 1, 57, 199):
        yp = h.matmul(np.ascontiguousarray(x[:, p]), device="cuda")
        assert np.array_equal(y[:, p], yp)
    yr = m.matmul(np.ascontiguousarray(x[:, :4]))
    assert rel_err(y[:, :4], yr) <= TOL


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_split_task_path_is_bitwise_equal(cuda_device, name, monkeypatch):
    """Every column task cut into one-chunk parts (QHMAT_GB300_PART_CHUNKS=1),
    so that every fixture with a task of two or more chunks runs the split
    path (64-bit atomic partial sums, fence, last-finisher counter): the
    integer sums are exact, so y equals the default layout's bit for bit."""
    data, g = golden(name)
    y_default = HMatrix.from_bytes(data).matmul(g["x"])
    monkeypatch.setenv("QHMAT_GB300_PART_CHUNKS", "1")
    h = HMatrix.from_bytes(data)
    y1 = h.matmul(g["x"])
    y2 = h.matmul(g["x"])
    assert np.array_equal(y1, y_default)
    assert np.array_equal(y1, y2)
    assert rel_err(y1, g["y"]) <= TOL


def test_wait_timeout_sets_status(cuda_device):
    """The bounded device wait gives up and reports QH_STATUS_TIMEOUT, which the
    host maps to QH_ERUNTIME; the context stays usable afterwards."""
    from qhmat_gb300 import _lib

    lib = _lib.load_library()
    rc = lib.qh_debug_wait_timeout(cuda_device, 64)
    assert rc == _lib.QH_ERUNTIME
    assert "device copy wait timed out" in lib.qh_last_error().decode()
    data, g = golden("cfg1")
    assert rel_err(HMatrix.from_bytes(data).matmul(g["x"]), g["y"]) <= TOL


def test_nonfinite_tensor_path_status(cuda_device):
    """A NaN or infinity in a device x sets QH_STATUS_NONFINITE in the status
    int (tensor path: ValueError; raw C ABI: the bit)."""
    import torch

    from qhmat_gb300 import _lib

    data, g = golden("cfg1")
    h = HMatrix.from_bytes(data)
    x = torch.from_numpy(g["x"].copy()).cuda()
    x[17, 2] = float("nan")
    with pytest.raises(ValueError, match="nonfinite right-hand side"):
        h.matmul(x)
    x[17, 2] = float("-inf")
    lib = _lib.load_library()
    y = torch.empty_like(x)
    need = h.workspace_bytes(4)
    ws = torch.empty(need, dtype=torch.uint8, device=x.device)
    status = torch.zeros(1, dtype=torch.int32, device=x.device)
    _lib.raise_for(lib.qh_matmul_device(h._h, x.data_ptr(), y.data_ptr(), 4, ws.data_ptr(), need,
                                        torch.cuda.current_stream().cuda_stream, status.data_ptr()))
    assert int(status.item()) == _lib.QH_STATUS_NONFINITE
    x[17, 2] = 0.5
    assert rel_err(h.matmul(x).cpu().numpy(), O.OracleMatrix(data).matmul(x.cpu().numpy())) <= TOL


def test_more_than_65535_columns(cuda_device):
    """An apply with 65539 right-hand sides (more than one launch grid's
    gridDim.y) runs in column chunks: every column equals its own apply bit for
    bit and the oracle within the tolerance (the reference accepts any rhs with
    order * rhs <= INT_MAX * 256, src/qhmat/cuda.cu:111-112)."""
    data, g = golden("cuda10")
    h = HMatrix.from_bytes(data)
    rhs = 65539
    x = np.random.default_rng(5).standard_normal((h.order, rhs))
    y = h.matmul(x)
    for p in (0, 65534, 65535, 65538):
        assert np.array_equal(y[:, p], h.matmul(np.ascontiguousarray(x[:, p])))
    assert rel_err(y, O.OracleMatrix(data).matmul(x)) <= TOL


def test_rhs_limits_match_reference(cuda_device):
    """rhs = 0 is a shape mismatch and order * rhs > INT_MAX * 256 is "CUDA launch
    grid too large", both raised before any device work
    (src/qhmat/cuda.cu:108-112)."""
    import ctypes as C

    from qhmat_gb300 import _lib

    data, _ = golden("cuda10")
    h = HMatrix.from_bytes(data)
    lib = _lib.load_library()
    dummy = np.zeros(4)
    p = dummy.ctypes.data_as(C.c_void_p)
    assert lib.qh_matmul_host(h._h, p, p, 0) == _lib.QH_EINVAL
    assert "right-hand-side shape mismatch" in lib.qh_last_error().decode()
    too_many = (2**31 - 1) * 256 // h.order + 1
    assert lib.qh_matmul_host(h._h, p, p, too_many) == _lib.QH_EOVERFLOW
    assert "CUDA launch grid too large" in lib.qh_last_error().decode()
    assert lib.qh_matmul_device(h._h, p, p, too_many, None, 0, None, None) == _lib.QH_EOVERFLOW


def test_cpu_device_is_rejected(cuda_device):
    """The reference's matmul defaults to device="cpu" (python/qhmat/matrix.py:
    295-303); this library applies on the GPU only and says so instead of
    falling back to a CPU loop."""
    data, g = golden("cuda10")
    h = HMatrix.from_bytes(data)
    with pytest.raises(ValueError, match="GPU only"):
        h.matmul(g["x"], device="cpu")
    with pytest.raises(RuntimeError, match="GPU only"):
        NativeHMatrix.from_bytes(data).matmul(g["x"], False)
