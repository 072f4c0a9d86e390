"""The CPU oracle pinned against the reference (CPU-only tests).

The oracle (oracle/qhmat_oracle.c) restates the reference's load / decode /
matmul / pack.  These tests pin it bit-for-bit against the golden fixtures made
by the reference (tests/golden/make_golden.py) and, where the reference's core
was compiled into oracle/_ref (build container only), against the reference
itself on fresh inputs.
"""

import numpy as np
import pytest

from conftest import GOLDEN_CASES, ROOT, golden
from oracle import oracle as O


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_oracle_matches_reference_matmul_bitwise(name):
    data, g = golden(name)
    m = O.OracleMatrix(data)
    y = m.matmul(g["x"])
    assert np.array_equal(y, g["y"]), "oracle matmul differs from the reference's"
    assert m.reconstruction_bound == float(g["bound"])
    if "dense" in g:
        assert np.array_equal(m.reconstruct(), g["dense"])


@pytest.mark.parametrize("name", ["cfg1", "ragged300", "cuda10"])
@pytest.mark.parametrize("threads", [2, 3, 8])
def test_threaded_oracle_is_bit_identical(name, threads):
    data, g = golden(name)
    m = O.OracleMatrix(data)
    assert np.array_equal(m.matmul(g["x"], threads=threads), g["y"])


def _pack_codes(codes: np.ndarray, w: int) -> np.ndarray:
    """Bit-pack signed integers LSB-first at width w (the reference's layout)."""
    rows = codes.size
    nwords = (rows * w + 31) // 32
    out = np.zeros(nwords + 1, np.uint64)
    raw = codes.astype(np.int64) & ((1 << w) - 1)
    pos = np.arange(rows, dtype=np.int64) * w
    for i in range(rows):
        word, shift = divmod(int(pos[i]), 32)
        v = int(raw[i]) << shift
        out[word] |= np.uint64(v & 0xFFFFFFFF)
        out[word + 1] |= np.uint64(v >> 32)
    return out[:nwords].astype(np.uint32)


def _file_words(data: bytes, m: "O.OracleMatrix"):
    """Re-read each low-rank block's word runs from a QHMAT001 image."""
    import struct

    n = m.order
    off = 8 + 8 * 3 + 8 * n
    out = []
    for b in range(m.block_count):
        info = m.block_info(b)
        rows, cols = info["row1"] - info["row0"], info["col1"] - info["col0"]
        off += 34
        if info["dense"]:
            off += 8 * rows * cols
            out.append(None)
            continue
        rank = info["rank"]
        off += 32 + rank + 16 * rank
        lw, rw = info["left_words"], info["right_words"]
        left = np.frombuffer(data, np.uint32, lw, off)
        right = np.frombuffer(data, np.uint32, rw, off + 4 * lw)
        off += 4 * (lw + rw)
        out.append((left, right))
    assert off == len(data) - 8
    return out


@pytest.mark.parametrize("name", ["ragged300", "cfg1", "orth17_b12", "orth17_b24", "kernel12"])
def test_decoded_codes_repack_to_the_stored_words(name):
    """Round trip: the oracle's decode, re-packed, reproduces every stored word."""
    data, _ = golden(name)
    m = O.OracleMatrix(data)
    words = _file_words(data, m)
    for b in range(m.block_count):
        info = m.block_info(b)
        if info["dense"] or info["rank"] == 0:
            continue
        widths = m.widths(b)
        for side, stored in ((0, words[b][0]), (1, words[b][1])):
            codes = m.codes(b, side)
            rebuilt = np.concatenate([_pack_codes(codes[j], int(widths[j])) for j in range(len(widths))])
            assert np.array_equal(rebuilt, stored), (b, side)
            q = (1 << (widths.astype(np.int64) - 1)) - 1
            assert np.all(np.abs(codes) <= q[:, None])


def test_oracle_pack_matches_reference_pack():
    """oracle pack == reference add_low_rank's packing on the same factors."""
    if not O.reference_available():
        pytest.skip("reference core not built here (oracle/_ref)")
    from oracle.build_ref import import_reference_qhmat

    q = import_reference_qhmat()
    import tempfile
    from pathlib import Path

    rng = np.random.default_rng(7)
    for bits in (2, 5, 12, 24, 31, 32):
        u, _ = np.linalg.qr(rng.normal(size=(37, 4)))
        v, _ = np.linalg.qr(rng.normal(size=(29, 4)))
        sigma = np.array([5.0, 2.0, 0.3, 0.01])
        native = q.NativeHMatrix(66, list(range(66)))
        native.add_dense(q.Rectangle(0, 37, 0, 37), np.eye(37))
        native.add_dense(q.Rectangle(37, 66, 37, 66), np.eye(29))
        native.add_low_rank(q.Rectangle(0, 37, 37, 66), u, sigma, v, [bits] * 4, 1, 0.0)
        native.add_low_rank(q.Rectangle(37, 66, 0, 37), v, sigma, u, [bits] * 4, 1, 0.0)
        native.finalize()
        with tempfile.TemporaryDirectory() as d:
            p = Path(d) / "m.qhmat"
            native.save(str(p))
            data = p.read_bytes()
        m = O.OracleMatrix(data)
        stored = _file_words(data, m)
        for b, (uu, vv) in ((2, (u, v)), (3, (v, u))):
            lw, _, _ = O.pack(uu * np.sqrt(sigma), [bits] * 4)
            rw, _, _ = O.pack(vv * np.sqrt(sigma), [bits] * 4)
            assert np.array_equal(lw, stored[b][0])
            assert np.array_equal(rw, stored[b][1])


def test_oracle_agrees_with_compiled_reference_on_fresh_inputs():
    if not O.reference_available():
        pytest.skip("reference core not built here (oracle/_ref)")
    for name in ("cfg1", "ragged300"):
        data, g = golden(name)
        ref = O.RefMatrix(data)
        m = O.OracleMatrix(data)
        x = np.random.default_rng(123).standard_normal((m.order, 5))
        assert np.array_equal(ref.matmul(x), m.matmul(x))
        assert np.array_equal(ref.matmul(x[:, 0]), m.matmul(x[:, 0], threads=4))


@pytest.mark.parametrize("mutate,match", [
    (lambda d: d[:-5], "truncated|trailing"),
    (lambda d: d[:-9] + bytes([d[-9] ^ 1]) + d[-8:], "checksum"),
    (lambda d: b"QHMAT002" + d[8:], "magic"),
    (lambda d: d[:16] + (0).to_bytes(8, "little") + d[24:], "dimensions"),
])
def test_oracle_rejects_corrupt_images(mutate, match):
    data, _ = golden("packed8")
    with pytest.raises(RuntimeError, match=match):
        O.OracleMatrix(mutate(data))


def test_oracle_rejects_nonfinite_rhs():
    data, g = golden("cuda10")
    m = O.OracleMatrix(data)
    x = g["x"].copy()
    x[3, 1] = np.nan
    with pytest.raises(ValueError, match="nonfinite"):
        m.matmul(x)


def test_oracle_checksum_matches_trailer():
    """The C restatement's FNV-1a-64 reproduces every fixture's trailer (the
    CPU baseline writes images with it, without loading the CUDA library)."""
    for name in ("tiny2", "cfg1", "ragged300"):
        data = (ROOT / "tests" / "golden" / f"{name}.qhmat").read_bytes()
        assert O.fnv1a64(data[:-8]) == int.from_bytes(data[-8:], "little")


def test_reference_arm_never_loads_the_cuda_library():
    """bench.py --impl reference on the n=2048 workload: one JSON line with the
    reference arm's fields and the same config keys as the GPU arm, and the
    process maps no libqhmat_gb300.so."""
    import json
    import subprocess
    import sys

    code = ("import sys, bench; sys.argv = ['bench.py', '--impl', 'reference', '--workload', 'cfg1', "
            "'--steps', '3', '--warmup', '3']; bench.main(); "
            "print('MAPS', open('/proc/self/maps').read().count('libqhmat_gb300'))")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.strip().splitlines()
    assert lines[-1] == "MAPS 0"
    out = json.loads(lines[-2])
    assert out["impl"] == "reference" and out["e2e"]["h2d_bytes_per_step"] == 0
    # the config is the workload alone (equal in both arms); timings sit outside it
    assert set(out["config"]) == {"workload", "n", "rhs", "tolerance", "tolerance_requested",
                                  "tolerance_note", "l2"}
    assert "construction_s" in out
