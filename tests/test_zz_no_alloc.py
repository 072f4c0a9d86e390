"""The allocation-free apply, qh_matmul_device_static, through the C ABI.

Some callers cannot allocate device memory while they apply a matrix: a
plugin whose host framework owns all device memory through its own
allocator, a latency-critical loop that cannot afford cudaMalloc's implicit
device synchronisation, or code held to a fixed pre-reserved memory budget.
For them qh_matmul_device_static uses a fixed static device array as its
scratch instead of a workspace.  This file checks that two calls in a row
give the same y as qh_matmul_device -- bit for bit, since both run the same
exact-integer kernels on the same inputs, so a stale-scratch fault that moved
even one low bit would show -- that an apply needing more scratch than the
array holds is rejected, and that the result still matches the reference
within the 1e-13 tolerance the other GPU tests use.  It runs last
(file name) so that a stop at the first failure has already run every other
test; it passes alone and after them.
"""

import ctypes as C

import numpy as np
import pytest

from conftest import golden, rel_err
from qhmat_gb300 import HMatrix, _lib

pytestmark = pytest.mark.gpu
TOL = 1e-13


def _apply_both(h, x_np):
    import torch

    lib = _lib.load_library()
    dev = torch.device("cuda", h.device)
    x = torch.from_numpy(np.ascontiguousarray(x_np)).to(dev)
    rhs = 1 if x.ndim == 1 else x.shape[1]
    stream = torch.cuda.current_stream(dev)
    need = h.workspace_bytes(rhs)
    ws = torch.empty(need, dtype=torch.uint8, device=dev)
    y_ref = torch.empty_like(x)
    _lib.raise_for(lib.qh_matmul_device(h._h, x.data_ptr(), y_ref.data_ptr(), rhs, ws.data_ptr(), need,
                                        stream.cuda_stream, None))
    outs = []
    for _ in range(2):  # two calls in a row share (and must clear) the static scratch
        y = torch.full_like(x, float("nan"))
        status = torch.zeros(1, dtype=torch.int32, device=dev)
        _lib.raise_for(lib.qh_matmul_device_static(h._h, x.data_ptr(), y.data_ptr(), rhs, stream.cuda_stream,
                                                   status.data_ptr()))
        torch.cuda.synchronize(dev)
        assert int(status.item()) == 0
        outs.append(y.cpu().numpy())
    return y_ref.cpu().numpy(), outs


@pytest.mark.parametrize("name", ["cfg1", "ragged300", "cuda10"])
def test_static_scratch_apply_matches_workspace_apply(cuda_device, name):
    data, g = golden(name)
    h = HMatrix.from_bytes(data, device=cuda_device)
    y_ref, outs = _apply_both(h, g["x"])
    for y in outs:
        assert np.array_equal(y, y_ref)
        assert rel_err(y, g["y"]) <= TOL


def test_static_scratch_apply_rejects_oversized_scratch(cuda_device):
    import torch

    data, _ = golden("cfg1")
    h = HMatrix.from_bytes(data, device=cuda_device)
    lib = _lib.load_library()
    limit = 16 << 20
    rhs = 1
    while h.workspace_bytes(rhs) <= limit:
        rhs *= 2
    dev = torch.device("cuda", cuda_device)
    x = torch.zeros((h.order, rhs), dtype=torch.float64, device=dev)
    y = torch.empty_like(x)
    rc = lib.qh_matmul_device_static(h._h, x.data_ptr(), y.data_ptr(), rhs,
                                     torch.cuda.current_stream(dev).cuda_stream, None)
    assert rc == _lib.QH_EINVAL
    assert "QH_STATIC_SCRATCH_BYTES" in lib.qh_last_error().decode()
