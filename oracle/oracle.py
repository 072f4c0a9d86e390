"""ctypes front end of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg import this module, and only as the checker.  Two back ends:

* :class:`OracleMatrix` -- the plain-C restatement ``oracle/qhmat_oracle.c``
  (compiled on whatever machine runs the tests, x86 or Arm);
* :class:`RefMatrix` -- the reference's own C++ core compiled from its sources
  into ``oracle/_ref/libqhmat_ref.so`` by ``oracle/build_ref.py`` (present only
  where the reference sources were available to build it).
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"
REF_LIB = HERE / "_ref" / "libqhmat_ref.so"

_lib = None
_ref = None


def build(force: bool = False) -> Path:
    """Compile qhmat_oracle.c with the host C compiler (portable C11, -O2).

    -ffp-contract=off keeps every a * b + c as a rounded multiply and a
    rounded add, as the reference's own x86-64 build evaluates them; aarch64
    compilers would otherwise fuse them into FMAs and change the last bit."""
    src = HERE / "qhmat_oracle.c"
    if force or not LIB.exists() or LIB.stat().st_mtime < src.stat().st_mtime:
        LIB.parent.mkdir(exist_ok=True)
        tmp = LIB.with_suffix(f".{os.getpid()}.tmp")
        subprocess.run(["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fPIC", "-shared", "-fvisibility=hidden",
                        "-D_GNU_SOURCE", str(src), "-o", str(tmp), "-lm", "-lpthread"],
                       check=True)
        os.replace(tmp, LIB)
    return LIB


def _load():
    global _lib
    if _lib is None:
        lib = C.CDLL(str(build()))
        lib.qho_parse.restype = C.c_void_p
        lib.qho_parse.argtypes = [C.c_char_p, C.c_uint64, C.c_char_p, C.c_size_t]
        lib.qho_free.argtypes = [C.c_void_p]
        lib.qho_order.restype = C.c_uint64
        lib.qho_order.argtypes = [C.c_void_p]
        lib.qho_block_count.restype = C.c_uint64
        lib.qho_block_count.argtypes = [C.c_void_p]
        lib.qho_block_info.argtypes = [C.c_void_p, C.c_uint64, C.c_void_p]
        lib.qho_block_widths.argtypes = [C.c_void_p, C.c_uint64, C.c_void_p]
        lib.qho_block_codes.argtypes = [C.c_void_p, C.c_uint64, C.c_int, C.c_void_p]
        lib.qho_fnv1a64.restype = C.c_uint64
        lib.qho_fnv1a64.argtypes = [C.c_char_p, C.c_uint64]
        lib.qho_bound.restype = C.c_double
        lib.qho_bound.argtypes = [C.c_void_p]
        lib.qho_matmul.restype = C.c_int
        lib.qho_matmul.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, C.c_int,
                                   C.c_char_p, C.c_size_t]
        lib.qho_reconstruct.argtypes = [C.c_void_p, C.c_void_p]
        lib.qho_pack.argtypes = [C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint64, C.c_void_p,
                                 C.c_void_p, C.c_void_p]
        _lib = lib
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


class OracleMatrix:
    """A QHMAT001 image parsed by the C restatement of the reference."""

    def __init__(self, data: bytes):
        lib = _load()
        err = C.create_string_buffer(512)
        h = lib.qho_parse(data, len(data), err, 512)
        if not h:
            raise RuntimeError(err.value.decode())
        self._h = h
        self._lib = lib

    @classmethod
    def load(cls, path) -> "OracleMatrix":
        return cls(Path(path).read_bytes())

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.qho_free(self._h)
            self._h = None

    @property
    def order(self) -> int:
        return int(self._lib.qho_order(self._h))

    @property
    def block_count(self) -> int:
        return int(self._lib.qho_block_count(self._h))

    @property
    def reconstruction_bound(self) -> float:
        return float(self._lib.qho_bound(self._h))

    def block_info(self, b: int) -> dict:
        out = np.zeros(10, np.uint64)
        self._lib.qho_block_info(self._h, b, _ptr(out))
        keys = ("row0", "row1", "col0", "col1", "admissible", "dense", "rank", "menu_size",
                "left_words", "right_words")
        return {k: int(v) for k, v in zip(keys, out)}

    def widths(self, b: int) -> np.ndarray:
        info = self.block_info(b)
        out = np.zeros(max(info["rank"], 1), np.uint8)
        self._lib.qho_block_widths(self._h, b, _ptr(out))
        return out[: info["rank"]]

    def codes(self, b: int, side: int) -> np.ndarray:
        """Decoded integer codes of one factor, shape (rank, rows)."""
        info = self.block_info(b)
        rows = (info["row1"] - info["row0"]) if side == 0 else (info["col1"] - info["col0"])
        out = np.zeros((info["rank"], rows), np.int32)
        if info["rank"]:
            self._lib.qho_block_codes(self._h, b, side, _ptr(out))
        return out

    def matmul(self, x: np.ndarray, threads: int = 1) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float64)
        if x.ndim not in (1, 2) or x.shape[0] != self.order:
            raise ValueError("right-hand side has the wrong shape")
        rhs = 1 if x.ndim == 1 else x.shape[1]
        y = np.empty_like(x)
        err = C.create_string_buffer(512)
        if self._lib.qho_matmul(self._h, _ptr(x), _ptr(y), rhs, threads, err, 512):
            raise ValueError(err.value.decode())
        return y

    def reconstruct(self) -> np.ndarray:
        n = self.order
        out = np.empty((n, n), np.float64)
        self._lib.qho_reconstruct(self._h, _ptr(out))
        return out


def pack(matrix: np.ndarray, widths) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """HMatrix::pack restated: column-major (rows, ncomp) -> words, offsets, scales."""
    m = np.asfortranarray(matrix, dtype=np.float64)
    rows, ncomp = m.shape
    w = np.ascontiguousarray(widths, dtype=np.int32)
    nwords = int(sum((rows * int(b) + 31) // 32 for b in w))
    words = np.zeros(max(nwords, 1), np.uint32)
    offsets = np.zeros(max(ncomp, 1), np.uint64)
    scales = np.zeros(max(ncomp, 1), np.float64)
    _load().qho_pack(m.ctypes.data_as(C.c_void_p), rows, _ptr(w), ncomp, _ptr(words),
                     _ptr(offsets), _ptr(scales))
    return words[:nwords], offsets[:ncomp], scales[:ncomp]


def fnv1a64(data: bytes) -> int:
    """QHMAT001 trailer checksum computed by the C restatement."""
    return int(_load().qho_fnv1a64(data, len(data)))


def reference_available() -> bool:
    """True when oracle/_ref holds a loadable build of the reference core."""
    try:
        _ref_lib()
        return True
    except OSError:
        return False


def _ref_lib():
    global _ref
    if _ref is None:
        lib = C.CDLL(str(REF_LIB))
        lib.qhref_load.restype = C.c_void_p
        lib.qhref_load.argtypes = [C.c_char_p, C.c_char_p, C.c_size_t]
        lib.qhref_free.argtypes = [C.c_void_p]
        lib.qhref_order.restype = C.c_size_t
        lib.qhref_order.argtypes = [C.c_void_p]
        lib.qhref_bound.restype = C.c_double
        lib.qhref_bound.argtypes = [C.c_void_p]
        lib.qhref_matmul.restype = C.c_int
        lib.qhref_matmul.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t,
                                     C.c_char_p, C.c_size_t]
        lib.qhref_reconstruct.restype = C.c_int
        lib.qhref_reconstruct.argtypes = [C.c_void_p, C.c_void_p, C.c_char_p, C.c_size_t]
        _ref = lib
    return _ref


class RefMatrix:
    """The reference's own HMatrix (io.cpp load, core.cpp matmul), via ctypes."""

    def __init__(self, data: bytes):
        lib = _ref_lib()
        fd, path = tempfile.mkstemp(suffix=".qhmat")
        try:
            with os.fdopen(fd, "wb") as f:
                f.write(data)
            err = C.create_string_buffer(512)
            h = lib.qhref_load(path.encode(), err, 512)
        finally:
            os.unlink(path)
        if not h:
            raise RuntimeError(err.value.decode())
        self._h = h
        self._lib = lib

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.qhref_free(self._h)
            self._h = None

    @property
    def order(self) -> int:
        return int(self._lib.qhref_order(self._h))

    @property
    def reconstruction_bound(self) -> float:
        return float(self._lib.qhref_bound(self._h))

    def matmul(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float64)
        rhs = 1 if x.ndim == 1 else x.shape[1]
        y = np.empty_like(x)
        err = C.create_string_buffer(512)
        if self._lib.qhref_matmul(self._h, _ptr(x), _ptr(y), rhs, err, 512):
            raise ValueError(err.value.decode())
        return y

    def reconstruct(self) -> np.ndarray:
        n = self.order
        out = np.empty((n, n), np.float64)
        err = C.create_string_buffer(512)
        if self._lib.qhref_reconstruct(self._h, _ptr(out), err, 512):
            raise ValueError(err.value.decode())
        return out
