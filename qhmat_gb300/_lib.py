"""ctypes binding of ``libqhmat_gb300.so`` (the C ABI in include/qhmat_gb300.h).

The library is the only compute path: if it is missing or fails to load, every
entry point raises instead of falling back to anything else.
"""

from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libqhmat_gb300.so"

QH_OK, QH_EINVAL, QH_ERUNTIME, QH_EOVERFLOW, QH_ECUDA = 0, 1, 2, 3, 4
# bits of the device-side status int (include/qhmat_gb300.h QH_STATUS_*)
QH_STATUS_NONFINITE, QH_STATUS_TIMEOUT = 1, 2


class QhStats(C.Structure):
    _fields_ = [(name, C.c_uint64) for name in (
        "order", "block_count", "dense_blocks", "lowrank_blocks", "components", "code_bytes",
        "scale_bytes", "dense_bytes", "model_bytes", "device_bytes", "row_tiles", "flops_per_rhs",
        "launches_per_apply", "host_direct", "left_code_bytes", "right_code_bytes")]


class QhPStats(C.Structure):
    _fields_ = [(name, C.c_uint64) for name in (
        "order", "components", "code_bytes", "scale_bytes", "dense_bytes", "stored_q_bytes",
        "stored_p_bytes", "stored_dense_bytes", "device_bytes", "col_items", "row_items", "row_slots",
        "mma_elements", "launches_per_pass", "mma_col_elements", "mma_row_elements", "segment_chunks")]


class QhBlockDesc(C.Structure):
    _fields_ = [("row0", C.c_size_t), ("row1", C.c_size_t), ("col0", C.c_size_t),
                ("col1", C.c_size_t), ("rank", C.c_size_t), ("factor_offset", C.c_size_t),
                ("dense_offset", C.c_size_t), ("is_dense", C.c_int)]


_lib = None


def load_library() -> C.CDLL:
    """Load the in-tree CUDA library (building it first if QHMAT_GB300_BUILD=1)."""
    global _lib
    if _lib is not None:
        return _lib
    if os.environ.get("QHMAT_GB300_BUILD") == "1" or not LIB_PATH.exists():
        from . import build as _build

        try:
            _build.build()
        except Exception as exc:  # noqa: BLE001 - re-raised with context
            raise RuntimeError(f"qhmat_gb300 CUDA library is not built and building it failed: {exc}")
    lib = C.CDLL(str(LIB_PATH))
    vp, sz, i32 = C.c_void_p, C.c_size_t, C.c_int
    lib.qh_last_error.restype = C.c_char_p
    lib.qh_last_error.argtypes = []
    lib.qh_cuda_built.restype = i32
    lib.qh_cuda_built.argtypes = []
    lib.qh_matrix_from_qhmat.restype = i32
    lib.qh_matrix_from_qhmat.argtypes = [C.c_char_p, sz, i32, C.POINTER(vp)]
    lib.qh_matrix_from_arrays.restype = i32
    lib.qh_matrix_from_arrays.argtypes = [sz, vp, sz, vp, vp, vp, vp, vp, vp, vp, vp, vp, i32,
                                          C.POINTER(vp)]
    lib.qh_matrix_destroy.restype = None
    lib.qh_matrix_destroy.argtypes = [vp]
    lib.qh_matrix_stats.restype = i32
    lib.qh_matrix_stats.argtypes = [vp, C.POINTER(QhStats)]
    lib.qh_matrix_reconstruction_bound.restype = C.c_double
    lib.qh_matrix_reconstruction_bound.argtypes = [vp]
    lib.qh_workspace_bytes.restype = sz
    lib.qh_workspace_bytes.argtypes = [vp, sz]
    lib.qh_matmul_device.restype = i32
    lib.qh_matmul_device.argtypes = [vp, vp, vp, sz, vp, sz, vp, vp]
    lib.qh_matmul_device_profiled.restype = i32
    lib.qh_matmul_device_profiled.argtypes = [vp, vp, vp, sz, vp, sz, vp, vp, vp]
    lib.qh_matmul_device_static.restype = i32
    lib.qh_matmul_device_static.argtypes = [vp, vp, vp, sz, vp, vp]
    lib.qh_matmul_host.restype = i32
    lib.qh_matmul_host.argtypes = [vp, vp, vp, sz]
    lib.qh_fnv1a64.restype = C.c_uint64
    lib.qh_fnv1a64.argtypes = [C.c_char_p, sz]
    lib.qh_debug_decode.restype = i32
    lib.qh_debug_decode.argtypes = [vp, i32, vp, sz, C.POINTER(sz)]
    lib.qh_pmatrix_from_qhmat.restype = i32
    lib.qh_pmatrix_from_qhmat.argtypes = [C.c_char_p, sz, i32, C.POINTER(vp)]
    lib.qh_pmatrix_destroy.restype = None
    lib.qh_pmatrix_destroy.argtypes = [vp]
    lib.qh_pmatrix_stats.restype = i32
    lib.qh_pmatrix_stats.argtypes = [vp, C.POINTER(QhPStats)]
    lib.qh_pworkspace_bytes.restype = sz
    lib.qh_pworkspace_bytes.argtypes = [vp, sz]
    lib.qh_pmatmul_device.restype = i32
    lib.qh_pmatmul_device.argtypes = [vp, vp, vp, sz, vp, sz, vp, vp]
    lib.qh_qhmat_device_bytes.restype = i32
    lib.qh_qhmat_device_bytes.argtypes = [C.c_char_p, sz, C.c_int, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
    lib.qh_pmatrix_set_segment_chunks.restype = i32
    lib.qh_pmatrix_set_segment_chunks.argtypes = [vp, C.c_int]
    lib.qh_pmatmul_host.restype = i32
    lib.qh_pmatmul_host.argtypes = [vp, vp, vp, sz]
    lib.qh_pmatrix_host_direct.restype = i32
    lib.qh_pmatrix_host_direct.argtypes = [vp]
    lib.qh_pmatmul_device_profiled.restype = i32
    lib.qh_pmatmul_device_profiled.argtypes = [vp, vp, vp, sz, vp, sz, vp, vp, vp]
    ll = C.c_longlong
    for name in ("qh_gather_columns", "qh_scatter_columns"):
        f = getattr(lib, name)
        f.restype = i32
        f.argtypes = [vp, ll, vp, ll, vp, i32, sz, vp]
    lib.qh_matrix_from_batch.restype = i32
    lib.qh_matrix_from_batch.argtypes = [vp, vp, sz, i32, C.POINTER(vp), vp]
    lib.qh_pmatrix_from_batch.restype = i32
    lib.qh_pmatrix_from_batch.argtypes = [vp, vp, sz, i32, i32, C.c_double, C.POINTER(vp), vp]
    lib.qh_batch_gather.restype = i32
    lib.qh_batch_gather.argtypes = [vp, sz, i32, vp, vp, vp, vp]
    lib.qh_batch_scatter.restype = i32
    lib.qh_batch_scatter.argtypes = [vp, sz, i32, vp, vp, vp, vp]
    lib.qh_debug_wait_timeout.restype = i32
    lib.qh_debug_wait_timeout.argtypes = [i32, i32]
    lib.qh_matrix_reconstruct.restype = i32
    lib.qh_matrix_reconstruct.argtypes = [vp, vp, sz, i32]
    _lib = lib
    return lib


def raise_for(code: int) -> None:
    """Map a QH_* status to the exception type the reference raises."""
    if code == QH_OK:
        return
    msg = load_library().qh_last_error().decode(errors="replace")
    if code == QH_EINVAL:
        raise ValueError(msg)
    if code == QH_EOVERFLOW:
        raise OverflowError(msg)
    raise RuntimeError(msg)
