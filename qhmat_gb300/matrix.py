"""GPU-resident drop-in for the reference's quantized H-matrix apply.

Mirrors ``qhmat.HMatrix.matmul(x, *, device="cuda")`` (python/qhmat/matrix.py:
295-303) and ``NativeHMatrix.matmul(x, use_cuda)`` (src/qhmat/bindings.cpp:
152-179): same argument meaning, same shape rules, same exception types and
messages.  The difference is residency: the representation is uploaded once
when the object is created, and every ``matmul`` only moves x and y.

Inputs may be NumPy arrays (host path: one pinned copy in and one copy out per
call, through ``qh_matmul_host``) or CUDA ``torch.float64`` tensors (device
path: zero-copy, stream-ordered, through ``qh_matmul_device``; the result is a
CUDA tensor).  Only the GPU applies: ``device="cpu"`` is rejected rather than
served by a CPU fallback.
"""

from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

from ._lib import QH_STATUS_NONFINITE, QH_STATUS_TIMEOUT, QhBlockDesc, QhPStats, QhStats, load_library, raise_for


def _torch():
    import torch

    return torch


def _is_torch_tensor(x) -> bool:
    mod = type(x).__module__
    return mod.startswith("torch") and hasattr(x, "is_cuda")


class HMatrix:
    """A quantized H-matrix resident on one CUDA device."""

    def __init__(self, handle: int, device: int):
        self._lib = load_library()
        self._h = C.c_void_p(handle)
        self._device = device
        st = QhStats()
        raise_for(self._lib.qh_matrix_stats(self._h, C.byref(st)))
        self._stats = {name: int(getattr(st, name)) for name, _ in QhStats._fields_}

    # ------------------------------------------------------------ creation
    @classmethod
    def from_bytes(cls, data: bytes, *, device: int = 0, precision: bool = False) -> "HMatrix":
        """Parse and upload a QHMAT001 image (the reference's file format).

        ``precision=True`` also uploads the precision form and calibrates the
        choice between the two forms (``form_choice``) for ``matmul(...,
        form="auto")``."""
        lib = load_library()
        out = C.c_void_p()
        raise_for(lib.qh_matrix_from_qhmat(bytes(data), len(data), device, C.byref(out)))
        h = cls(out.value, device)
        if precision:
            h.attach_precision(PrecisionHMatrix.from_bytes(data, device=device))
        return h

    def attach_precision(self, pf: "PrecisionHMatrix", **calibration) -> dict:
        """Attach a precision-form handle of the same matrix and calibrate the
        form used by ``matmul(..., form="auto")`` for two or more columns."""
        self._pf = pf
        self.form_choice = choose_form(self, pf, **calibration)
        return self.form_choice

    @classmethod
    def load(cls, path: str | os.PathLike[str], *, device: int = 0) -> "HMatrix":
        """Load a file written by the reference's ``HMatrix.save``."""
        return cls.from_bytes(Path(path).read_bytes(), device=device)

    @classmethod
    def from_reference(cls, matrix, *, device: int = 0) -> "HMatrix":
        """Upload a reference ``qhmat.HMatrix`` / ``NativeHMatrix`` via its own ``save``."""
        import tempfile

        with tempfile.TemporaryDirectory() as d:
            path = Path(d) / "matrix.qhmat"
            matrix.save(str(path))
            return cls.load(path, device=device)

    @classmethod
    def from_arrays(cls, order, permutation, blocks, dense, left_words, right_words,
                    left_offsets, right_offsets, left_scales, right_scales, widths, *,
                    device: int = 0) -> "HMatrix":
        """Create from the flat arrays the reference's CUDA path builds per call.

        ``blocks`` is a sequence of (row0, row1, col0, col1, rank, factor_offset,
        dense_offset, is_dense) tuples (DeviceBlock, src/qhmat/cuda.cu:42-46).
        """
        lib = load_library()
        perm = np.ascontiguousarray(permutation, dtype=np.uintp)
        descs = (QhBlockDesc * len(blocks))(*[QhBlockDesc(*map(int, b)) for b in blocks])
        arrs = [np.ascontiguousarray(dense, np.float64), np.ascontiguousarray(left_words, np.uint32),
                np.ascontiguousarray(right_words, np.uint32),
                np.ascontiguousarray(left_offsets, np.uintp),
                np.ascontiguousarray(right_offsets, np.uintp),
                np.ascontiguousarray(left_scales, np.float64),
                np.ascontiguousarray(right_scales, np.float64), np.ascontiguousarray(widths, np.intc)]
        out = C.c_void_p()
        raise_for(lib.qh_matrix_from_arrays(order, perm.ctypes.data, len(blocks), C.addressof(descs),
                                            *[a.ctypes.data for a in arrs], device, C.byref(out)))
        return cls(out.value, device)

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            self._lib.qh_matrix_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001 - interpreter shutdown
            pass

    # ------------------------------------------------------------ metadata
    @property
    def order(self) -> int:
        return self._stats["order"]

    @property
    def shape(self) -> tuple[int, int]:
        return self.order, self.order

    @property
    def device(self) -> int:
        return self._device

    @property
    def reconstruction_bound(self) -> float:
        """Max-norm bound of the stored matrix (as the reference reports it)."""
        return float(self._lib.qh_matrix_reconstruction_bound(self._h))

    @property
    def stats(self) -> dict:
        """Block counts and the packed-byte traffic model of one apply."""
        return dict(self._stats)

    def model_bytes(self, rhs: int = 1) -> int:
        """Packed-byte traffic model of one apply with ``rhs`` columns."""
        s = self._stats
        return s["code_bytes"] + s["scale_bytes"] + s["dense_bytes"] + 16 * s["order"] * rhs

    def workspace_bytes(self, rhs: int = 1) -> int:
        return int(self._lib.qh_workspace_bytes(self._h, rhs))

    # ------------------------------------------------------------ apply
    def _check_shape(self, shape) -> int:
        if len(shape) not in (1, 2):
            raise ValueError("right-hand side must be one- or two-dimensional")
        if shape[0] != self.order:
            raise ValueError("right-hand side has the wrong row count")
        return 1 if len(shape) == 1 else int(shape[1])

    def matmul(self, x, *, device: str = "cuda", stream=None, workspace=None, check: bool = True,
               form: str = "plain"):
        """Apply to an ``(n,)`` vector or ``(n, p)`` array in FP64 on the GPU.

        NumPy input returns a new NumPy array; a CUDA float64 torch tensor
        returns a CUDA tensor computed on ``stream`` (default: torch's current
        stream).  ``check=False`` skips the device-side nonfinite check's host
        synchronisation on the tensor path.  ``form``: "plain" (default; the
        reference's result to ~1e-15), "precision" (the attached precision
        form), or "auto" (the precision form for two or more columns when the
        calibration chose it, else plain).
        """
        if device not in ("cpu", "cuda"):
            raise ValueError("device must be 'cpu' or 'cuda'")
        if device != "cuda":
            raise ValueError("qhmat_gb300 applies on the GPU only; use device='cuda'")
        if form not in ("plain", "precision", "auto"):
            raise ValueError("form must be 'plain', 'precision' or 'auto'")
        if form != "plain":
            pf = getattr(self, "_pf", None)
            if pf is None:
                raise ValueError("no precision form attached (create with precision=True)")
            shape = tuple(x.shape) if hasattr(x, "shape") else np.shape(x)
            rhs = 1 if len(shape) == 1 else int(shape[1])
            if form == "precision" or (rhs >= 2 and self.form_choice["form"] == "precision"):
                return pf.matmul(x, stream=stream, check=check)
        if _is_torch_tensor(x):
            return self._matmul_tensor(x, stream=stream, workspace=workspace, check=check)
        a = np.ascontiguousarray(np.asarray(x, dtype=np.float64))
        rhs = self._check_shape(a.shape)
        y = np.empty_like(a)
        raise_for(self._lib.qh_matmul_host(self._h, a.ctypes.data, y.ctypes.data, rhs))
        return y

    def _matmul_tensor(self, x, *, stream=None, workspace=None, check=True):
        torch = _torch()
        if not x.is_cuda or x.device.index != self._device:
            raise ValueError(f"tensor right-hand side must live on cuda:{self._device}")
        if x.dtype != torch.float64:
            raise ValueError("tensor right-hand side must be torch.float64")
        rhs = self._check_shape(tuple(x.shape))
        x = x.contiguous()
        y = torch.empty_like(x)
        need = self.workspace_bytes(rhs)
        if workspace is None:
            workspace = torch.empty(need, dtype=torch.uint8, device=x.device)
        elif workspace.numel() * workspace.element_size() < need:
            raise ValueError("workspace too small")
        status = torch.zeros(1, dtype=torch.int32, device=x.device)
        s = stream if stream is not None else torch.cuda.current_stream(x.device)
        raise_for(self._lib.qh_matmul_device(self._h, x.data_ptr(), y.data_ptr(), rhs,
                                             workspace.data_ptr(), need, s.cuda_stream,
                                             status.data_ptr()))
        if check:
            st = int(status.item())
            if st & QH_STATUS_NONFINITE:
                raise ValueError("nonfinite right-hand side")
            if st & QH_STATUS_TIMEOUT:
                raise RuntimeError("device copy wait timed out")
        return y

    def __matmul__(self, x):
        return self.matmul(x)

    def to_dense(self) -> np.ndarray:
        """The represented matrix as a dense FP64 array in source order, built on
        the GPU; equal bit for bit to ``qhmat.HMatrix.to_dense``
        (python/qhmat/matrix.py:309-311)."""
        n = self.order
        out = np.empty((n, n), np.float64)
        raise_for(self._lib.qh_matrix_reconstruct(self._h, out.ctypes.data, out.size, 0))
        return out

    def debug_decode(self, side: int) -> np.ndarray:
        """All codes of one factor side decoded on the GPU (component-major)."""
        need = C.c_size_t()
        raise_for(self._lib.qh_debug_decode(self._h, side, None, 0, C.byref(need)))
        out = np.empty(need.value, np.int32)
        raise_for(self._lib.qh_debug_decode(self._h, side, out.ctypes.data, out.size, None))
        return out


class NativeHMatrix(HMatrix):
    """Mirror of ``qhmat.NativeHMatrix.matmul(x, use_cuda)`` for the GPU apply."""

    def matmul(self, x, use_cuda: bool = True, **kw):  # type: ignore[override]
        if not use_cuda:
            raise RuntimeError("qhmat_gb300 applies on the GPU only; pass use_cuda=True")
        return super().matmul(x, device="cuda", **kw)

    def reconstruct(self) -> np.ndarray:
        """``NativeHMatrix.reconstruct()`` (src/qhmat/bindings.cpp:180-190): the
        dense matrix, flattened row-major."""
        return self.to_dense().reshape(-1)


class PrecisionHMatrix:
    """The precision form of a resident quantized H-matrix: many right-hand
    sides per pass over the codes on the tcgen05 tensor cores (f16 digit
    planes x hi/mid/lo f16 limbs, FP32 accumulation, FP64 scales, dense
    diagonal limbs and final sums).  Same apply contract as
    ``HMatrix.matmul``; results carry FP32-level rounding, so callers check
    them with :func:`precision_gate` against the plain form where they need a
    stated bound."""

    def __init__(self, handle: int, device: int):
        self._lib = load_library()
        self._h = C.c_void_p(handle)
        self._device = device
        st = QhPStats()
        raise_for(self._lib.qh_pmatrix_stats(self._h, C.byref(st)))
        self._stats = {name: int(getattr(st, name)) for name, _ in QhPStats._fields_}

    @classmethod
    def from_bytes(cls, data: bytes, *, device: int = 0) -> "PrecisionHMatrix":
        lib = load_library()
        out = C.c_void_p()
        raise_for(lib.qh_pmatrix_from_qhmat(bytes(data), len(data), device, C.byref(out)))
        return cls(out.value, device)

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            self._lib.qh_pmatrix_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001 - interpreter shutdown
            pass

    @property
    def order(self) -> int:
        return self._stats["order"]

    @property
    def stats(self) -> dict:
        return dict(self._stats)

    def workspace_bytes(self, rhs: int) -> int:
        return int(self._lib.qh_pworkspace_bytes(self._h, rhs))

    @property
    def segment_chunks(self) -> int:
        """K chunks per FP32 accumulation segment: 2 (default, faster) or 1
        (half the error: the tensor cores truncate as they accumulate)."""
        return self._stats["segment_chunks"]

    @segment_chunks.setter
    def segment_chunks(self, chunks: int) -> None:
        raise_for(self._lib.qh_pmatrix_set_segment_chunks(self._h, int(chunks)))
        self._stats["segment_chunks"] = int(chunks)

    @property
    def host_direct(self) -> bool:
        """True when NumPy applies read x and write y in host memory in place
        (the device walks the host's page tables), False when staged."""
        return bool(self._lib.qh_pmatrix_host_direct(self._h))

    def matmul(self, x, *, stream=None, workspace=None, check: bool = True):
        """Apply to ``(n,)`` or ``(n, p)`` FP64 input (NumPy: through
        ``qh_pmatmul_host``, a new NumPy result; CUDA torch tensor: on
        ``stream``, result a tensor)."""
        if not _is_torch_tensor(x):
            a = np.ascontiguousarray(np.asarray(x, dtype=np.float64))
            if a.ndim not in (1, 2):
                raise ValueError("right-hand side must be one- or two-dimensional")
            if a.shape[0] != self.order:
                raise ValueError("right-hand side has the wrong row count")
            rhs = 1 if a.ndim == 1 else int(a.shape[1])
            y = np.empty_like(a)
            if a.size:
                raise_for(self._lib.qh_pmatmul_host(self._h, a.ctypes.data, y.ctypes.data, rhs))
            return y
        torch = _torch()
        xt = x
        if not xt.is_cuda or xt.device.index != self._device:
            raise ValueError(f"tensor right-hand side must live on cuda:{self._device}")
        if xt.dtype != torch.float64:
            raise ValueError("tensor right-hand side must be torch.float64")
        shape = tuple(xt.shape)
        if len(shape) not in (1, 2):
            raise ValueError("right-hand side must be one- or two-dimensional")
        if shape[0] != self.order:
            raise ValueError("right-hand side has the wrong row count")
        rhs = 1 if len(shape) == 1 else int(shape[1])
        xt = xt.contiguous()
        y = torch.empty_like(xt)
        need = self.workspace_bytes(rhs)
        if workspace is None:
            workspace = torch.empty(need, dtype=torch.uint8, device=xt.device)
        elif workspace.numel() * workspace.element_size() < need:
            raise ValueError("workspace too small")
        status = torch.zeros(1, dtype=torch.int32, device=xt.device)
        s = stream if stream is not None else torch.cuda.current_stream(xt.device)
        raise_for(self._lib.qh_pmatmul_device(self._h, xt.data_ptr(), y.data_ptr(), rhs, workspace.data_ptr(),
                                              need, s.cuda_stream, status.data_ptr()))
        if check:
            st = int(status.item())
            if st & QH_STATUS_NONFINITE:
                raise ValueError("nonfinite right-hand side")
            if st & QH_STATUS_TIMEOUT:
                raise RuntimeError("device copy wait timed out")
        return y


def precision_gate(y_form, y_plain, x, bound: float) -> dict:
    """The precision form's acceptance test against the plain form, per
    right-hand-side column: max_i |y_form - y_plain| <= 0.01 * bound * ||x||_1
    (the matrix's max-norm reconstruction bound scaled by the column's l1
    norm, the unit-consistent reading of "1% of reconstruction_bound").
    Returns the worst column's ratio (pass: <= 1) and both error figures."""
    yf = np.asarray(y_form, np.float64)
    yp = np.asarray(y_plain, np.float64)
    xx = np.asarray(x, np.float64)
    if yf.ndim == 1:
        yf, yp, xx = yf[:, None], yp[:, None], xx[:, None]
    dev = np.max(np.abs(yf - yp), axis=0)
    limit = 0.01 * bound * np.sum(np.abs(xx), axis=0)
    ratio = np.where(limit > 0, dev / np.where(limit > 0, limit, 1.0), np.where(dev > 0, np.inf, 0.0))
    return {"max_abs_dev": float(dev.max()), "worst_ratio": float(ratio.max()),
            "rel_err": float(np.linalg.norm(yf - yp) / max(np.linalg.norm(yp), 1e-300)),
            "passes": bool(ratio.max() <= 1.0)}


def choose_form(plain: "HMatrix", pf: PrecisionHMatrix, *, probes: int = 8, margin: float = 0.5,
                seed: int = 20240611) -> dict:
    """Pick the form for multi-right-hand-side applies of one matrix: apply both
    forms to ``probes`` seeded N(0, 1) columns and choose the precision form
    when the worst column's gate ratio (see :func:`precision_gate`) is at most
    ``margin`` -- a calibration, since the FP32 rounding of the precision
    form scales with the data and the gate with the matrix's bound.  The
    precision form is tried with two-chunk accumulation segments, then, if
    that misses the margin, with one-chunk segments (half the error, ~4% more
    time); the handle keeps the setting that passed (two when neither did)."""
    x = np.random.default_rng(seed).standard_normal((plain.order, probes))
    y_plain = plain.matmul(x)
    gate = precision_gate(pf.matmul(x), y_plain, x, plain.reconstruction_bound)
    if gate["worst_ratio"] > margin:
        pf.segment_chunks = 1
        fine = precision_gate(pf.matmul(x), y_plain, x, plain.reconstruction_bound)
        if fine["worst_ratio"] <= margin:
            gate = fine
        else:
            pf.segment_chunks = 2
    gate["form"] = "precision" if gate["worst_ratio"] <= margin else "plain"
    gate["segment_chunks"] = pf.segment_chunks
    gate["margin"] = margin
    return gate


def qhmat_device_bytes(data: bytes, *, sms: int, precision: bool = True) -> tuple[int, int]:
    """(plain-form, precision-form) device bytes of a QHMAT001 image's
    resident arenas, computed on the host without a device (the precision
    form's for a device of ``sms`` multiprocessors; 0 when ``precision`` is
    False).  Raises as ``HMatrix.from_bytes`` does for a corrupt image."""
    lib = load_library()
    plain, pf = C.c_uint64(), C.c_uint64()
    raise_for(lib.qh_qhmat_device_bytes(bytes(data), len(data), int(sms), C.byref(plain),
                                        C.byref(pf) if precision else None))
    return int(plain.value), int(pf.value) if precision else 0


def cuda_built() -> bool:
    return bool(load_library().qh_cuda_built())
