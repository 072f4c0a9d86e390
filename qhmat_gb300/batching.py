"""Batching form: many independent H-matrices applied in one graph launch.

The reference applies one matrix per call.  Here a set of matrices (each
with its own number of right-hand-side columns) is made resident as the
block-diagonal matrix diag(A_1, .., A_M): one plain-form handle and/or one
precision-form handle (``qh_matrix_from_batch`` / ``qh_pmatrix_from_batch``),
whose persistent column and row kernels walk the blocks of every matrix --
uneven sizes, ranks and widths -- in one launch each.  Each apply is:

  gather   the packed right-hand sides -> the block-diagonal operand, every
           column of every matrix scaled by a power of two (exact) so that
           all matrices keep full precision under the per-column exponents;
  apply    the precision-form batch (matrices whose calibration chose it) and
           the plain-form batch (the others), on two streams;
  scatter  the result columns back, scaled back exactly;

and the whole sequence is captured once as a CUDA graph, so an apply is one
graph launch.

Per-matrix form choice: each matrix is calibrated (both forms on seeded
probe columns, the acceptance gate of :func:`precision_gate`).  The precision
batch's schedule -- persistent CTAs and row items per CTA -- is chosen by a
small autotuner that times candidate schedules and caches the winner in a
JSON file under a key of the batch's right-hand-side count, dominant code
width and mean rank (buckets).  The MMA tile shape itself is fixed (M = 128,
K = 64 per chunk, N = 3p).
"""

from __future__ import annotations

import ctypes as C
import json
import os
import time
from pathlib import Path

import numpy as np

from ._lib import QhPStats, QhStats, load_library, raise_for
from .matrix import precision_gate


class BatchEntry(C.Structure):
    _fields_ = [(k, C.c_uint64) for k in ("offset", "order", "rows", "rhs", "x_offset", "y_offset")]


def _packed_offsets(orders, rhs):
    x_off = np.concatenate([[0], np.cumsum(np.asarray(orders, np.int64) * np.asarray(rhs, np.int64))])
    return x_off


class _Batch:
    """One block-diagonal handle (plain or precision) over a subset of the
    matrices, with its device table, operand buffers and workspace."""

    def __init__(self, images, orders, rhs, x_offs, device, precision, grid=0, row_items=0.0, seg=2):
        import torch

        self.lib = load_library()
        self.precision = precision
        self.count = len(images)
        self.P = int(max(rhs))
        bufs = [C.create_string_buffer(bytes(b), len(b)) for b in images]
        ptrs = (C.c_void_p * self.count)(*[C.addressof(b) for b in bufs])
        lens = (C.c_size_t * self.count)(*[len(b) for b in images])
        offs = (C.c_uint64 * self.count)()
        h = C.c_void_p()
        if precision:
            raise_for(self.lib.qh_pmatrix_from_batch(ptrs, lens, self.count, device, int(grid), float(row_items),
                                                     C.byref(h), offs))
            raise_for(self.lib.qh_pmatrix_set_segment_chunks(h, int(seg)))
        else:
            raise_for(self.lib.qh_matrix_from_batch(ptrs, lens, self.count, device, C.byref(h), offs))
        self.h = h
        self.offsets = list(offs)
        # the handle's order (the plain batch has no padding rows; the
        # precision batch starts every matrix on a multiple of 128 rows)
        if precision:
            st = QhPStats()
            raise_for(self.lib.qh_pmatrix_stats(h, C.byref(st)))
        else:
            st = QhStats()
            raise_for(self.lib.qh_matrix_stats(h, C.byref(st)))
        n_super = max(int(st.order), self.offsets[-1] + orders[-1])
        tab = (BatchEntry * self.count)()
        for k in range(self.count):
            nxt = self.offsets[k + 1] if k + 1 < self.count else n_super
            tab[k] = BatchEntry(self.offsets[k], orders[k], nxt - self.offsets[k], rhs[k], x_offs[k], x_offs[k])
        dev = torch.device("cuda", device)
        self.table = torch.frombuffer(bytearray(bytes(tab)), dtype=torch.uint8).to(dev)
        self.xs = torch.zeros(n_super * self.P, dtype=torch.float64, device=dev)
        self.ys = torch.zeros_like(self.xs)
        self.exps = torch.zeros(self.count * self.P, dtype=torch.int32, device=dev)
        if precision:
            need = self.lib.qh_pworkspace_bytes(h, self.P)
        else:
            need = self.lib.qh_workspace_bytes(h, self.P)
        self.ws = torch.empty(max(int(need), 256), dtype=torch.uint8, device=dev)
        self.need = int(need)
        self.n_super = n_super

    def apply(self, x_all, y_all, stream) -> None:
        lib, s = self.lib, stream.cuda_stream
        raise_for(lib.qh_batch_gather(self.table.data_ptr(), self.count, self.P, x_all.data_ptr(), self.xs.data_ptr(),
                                      self.exps.data_ptr(), s))
        if self.precision:
            raise_for(lib.qh_pmatmul_device(self.h, self.xs.data_ptr(), self.ys.data_ptr(), self.P,
                                            self.ws.data_ptr(), self.need, s, None))
        else:
            raise_for(lib.qh_matmul_device(self.h, self.xs.data_ptr(), self.ys.data_ptr(), self.P,
                                           self.ws.data_ptr(), self.need, s, None))
        raise_for(lib.qh_batch_scatter(self.table.data_ptr(), self.count, self.P, self.ys.data_ptr(),
                                       self.exps.data_ptr(), y_all.data_ptr(), s))

    def close(self):
        if self.h and self.h.value:
            (self.lib.qh_pmatrix_destroy if self.precision else self.lib.qh_matrix_destroy)(self.h)
            self.h = C.c_void_p()


def batch_forms(ratio2, ratio1, rhs, margin: float = 0.5):
    """The precision batch's segment length and each matrix's form, from the
    calibration's worst-column gate ratios with two-chunk (``ratio2``) and
    one-chunk (``ratio1``) accumulation segments: one-chunk segments for the
    whole precision batch when some matrix passes only with them, and then
    every matrix judged at that setting; a matrix with fewer than two columns
    stays plain (the precision form serves multi-column applies)."""
    need_fine = any(r2 > margin and r1 <= margin and p >= 2 for r2, r1, p in zip(ratio2, ratio1, rhs))
    seg = 1 if need_fine else 2
    ratios = ratio1 if seg == 1 else ratio2
    return seg, ["precision" if r <= margin and p >= 2 else "plain" for r, p in zip(ratios, rhs)]


def _bucket(v, edges):
    for e in edges:
        if v <= e:
            return e
    return edges[-1]


class BatchedHMatrices:
    """M independent matrices (QHMAT001 images) with rhs[k] columns each,
    applied together.  ``x_all`` / ``y_all``: device float64 tensors holding
    every matrix's x / y packed (matrix k's order_k x rhs_k row-major block at
    ``x_offsets[k]``).  ``forms``: "auto" (per-matrix calibration), "plain"
    or "precision"."""

    def __init__(self, images, rhs, *, device: int = 0, forms: str = "auto", autotune: bool = True,
                 cache: str | os.PathLike | None = None, calibration_probes: int = 4):
        import torch

        from .matrix import HMatrix

        self.device = device
        self.rhs = [int(r) for r in rhs]
        self.orders = []
        self.bounds = []
        for img in images:
            n = int.from_bytes(img[16:24], "little")
            self.orders.append(n)
        self.x_offsets = _packed_offsets(self.orders, self.rhs)
        self.total = int(self.x_offsets[-1])
        dev = torch.device("cuda", device)
        self.dev = dev
        self.streams = (torch.cuda.Stream(device=dev), torch.cuda.Stream(device=dev))
        self.form = ["plain"] * len(images)
        self.calibration = []
        self.pf_seg = 2  # accumulation segment of the precision batch (1 where a matrix needs it)
        # per-matrix reconstruction bounds (for the gate) from the plain handles' metadata
        self.stats = []
        for img in images:
            h = HMatrix.from_bytes(img, device=device)
            self.bounds.append(h.reconstruction_bound)
            self.stats.append(h.stats)
            h.close()
        if forms == "precision":
            self.form = ["precision"] * len(images)
        elif forms == "auto":
            self.form = self._calibrate(images, calibration_probes)
        self.tuning = None
        pf_idx = [k for k, f in enumerate(self.form) if f == "precision"]
        pl_idx = [k for k, f in enumerate(self.form) if f == "plain"]
        self.batches = []
        if pf_idx:
            params = {"grid": 0, "row_items": 0.0}
            if autotune:
                params = self._autotune(pf_idx, images, cache)
            self.batches.append(self._make(images, pf_idx, True, seg=self.pf_seg, **params))
        # plain matrices in sub-batches by right-hand-side count: the plain
        # form's work grows with the columns it is given (every matrix of a
        # sub-batch is applied to its widest column count), so a 3-column
        # matrix should not ride in a 32-column operand; these edges pad
        # uniform 1..32-column requests by ~14% (4/8/16/32 edges: ~30%)
        edges = (0, 2, 4, 6, 8, 12, 16, 24, 32, 1 << 30)
        for lo, hi in zip(edges[:-1], edges[1:]):
            sub = [k for k in pl_idx if lo < self.rhs[k] <= hi]
            if sub:
                self.batches.append(self._make(images, sub, False))
        while len(self.streams) < len(self.batches):
            self.streams = self.streams + (torch.cuda.Stream(device=dev),)
        self.graph = None

    # ------------------------------------------------------------ building
    def _make(self, images, idx, precision, grid=0, row_items=0.0, seg=2):
        return _Batch([images[k] for k in idx], [self.orders[k] for k in idx], [self.rhs[k] for k in idx],
                      [int(self.x_offsets[k]) for k in idx], self.device, precision, grid, row_items, seg)

    def _probe(self, probes):
        import torch

        x = torch.empty(self.total, dtype=torch.float64, device=self.dev)
        rng = np.random.default_rng(20240611)
        x.copy_(torch.from_numpy(rng.standard_normal(self.total)))
        return x

    def _calibrate(self, images, probes):
        """Both forms over the whole batch on seeded N(0,1) right-hand sides
        (the precision form with two-chunk and with one-chunk accumulation
        segments); a matrix takes the precision form when its worst column's
        gate ratio is at most 0.5.  The precision batch uses one-chunk
        segments when a matrix passes only with them (half the error, ~4%
        more time), and every matrix is then judged at that setting."""
        import torch

        idx = list(range(len(images)))
        x = self._probe(probes)
        outs = []
        for precision, seg in ((False, 2), (True, 2), (True, 1)):
            b = self._make(images, idx, precision, seg=seg)
            y = torch.zeros_like(x)
            b.apply(x, y, torch.cuda.current_stream(self.dev))
            torch.cuda.synchronize(self.dev)
            outs.append(y.cpu().numpy())
            b.close()
        xh = x.cpu().numpy()
        ratios = {2: [], 1: []}
        for k in idx:
            a, b_ = int(self.x_offsets[k]), int(self.x_offsets[k + 1])
            shape = (self.orders[k], self.rhs[k])
            for seg, y in ((2, outs[1]), (1, outs[2])):
                g = precision_gate(y[a:b_].reshape(shape), outs[0][a:b_].reshape(shape), xh[a:b_].reshape(shape),
                                   self.bounds[k])
                ratios[seg].append(g["worst_ratio"])
        self.pf_seg, forms = batch_forms(ratios[2], ratios[1], self.rhs)
        self.calibration = ratios[self.pf_seg]
        return forms

    def _autotune(self, idx, all_images, cache):
        """Time candidate schedules of the precision batch (persistent CTAs x
        row items per CTA) and keep the fastest; results cached in JSON under
        (rhs bucket, dominant width, rank bucket)."""
        import torch

        images = [all_images[k] for k in idx]
        rhs = [self.rhs[k] for k in idx]
        orders = [self.orders[k] for k in idx]
        key = self._tune_key(idx, rhs) + f"-s{self.pf_seg}"
        path = Path(cache) if cache else Path(os.environ.get("QHMAT_GB300_AUTOTUNE",
                                                             Path.home() / ".cache" / "qhmat_gb300" / "autotune.json"))
        table = {}
        if path.exists():
            try:
                table = json.loads(path.read_text())
            except ValueError:
                table = {}
        if key in table:
            self.tuning = dict(table[key], key=key, cached=True)
            return {"grid": table[key]["grid"], "row_items": table[key]["row_items"]}
        sms = torch.cuda.get_device_properties(self.dev).multi_processor_count
        x = self._probe(1)
        y = torch.zeros_like(x)
        x_offs = _packed_offsets(orders, rhs)
        results = []
        for grid in (sms, sms // 2):
            for row_items in (3.0, 6.0):
                b = _Batch(images, orders, rhs, [int(v) for v in x_offs[:-1]], self.device, True, grid, row_items,
                           self.pf_seg)
                s = torch.cuda.current_stream(self.dev)
                for _ in range(2):
                    b.apply(x, y, s)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(s)
                for _ in range(5):
                    b.apply(x, y, s)
                e1.record(s)
                torch.cuda.synchronize(self.dev)
                results.append({"grid": grid, "row_items": row_items, "ms": e0.elapsed_time(e1) / 5})
                b.close()
        best = min(results, key=lambda r: r["ms"])
        table[key] = {"grid": best["grid"], "row_items": best["row_items"], "ms": best["ms"], "candidates": results}
        try:
            path.parent.mkdir(parents=True, exist_ok=True)
            path.write_text(json.dumps(table, indent=1))
        except OSError:
            pass
        self.tuning = dict(table[key], key=key, cached=False)
        return {"grid": best["grid"], "row_items": best["row_items"]}

    def _tune_key(self, idx, rhs):
        """(rhs bucket, dominant code width, mean-rank bucket) of the matrices
        ``idx``: mean bits per code = packed code bytes / sum r(m+n), mean
        rank = components / low-rank blocks (from the handles' statistics)."""
        bits = sum(self.stats[k]["code_bytes"] * 8 for k in idx)
        entries = sum(self.stats[k]["flops_per_rhs"] // 2 - self.stats[k]["dense_bytes"] // 8 for k in idx)
        comps = sum(self.stats[k]["components"] for k in idx)
        blocks = sum(self.stats[k]["lowrank_blocks"] for k in idx)
        width = _bucket(bits / max(entries, 1), (4, 8, 12, 16, 24, 32))
        rank = _bucket(comps / max(blocks, 1), (4, 8, 16, 32, 64, 128, 1 << 30))
        return f"p{_bucket(max(rhs), (8, 16, 32, 64))}-w{width}-r{rank}"

    # ------------------------------------------------------------ apply
    def apply(self, x_all, y_all) -> None:
        """y_all = the batch applied to x_all (device tensors), on two streams
        joined to the current one."""
        import torch

        cur = torch.cuda.current_stream(self.dev)
        for b, s in zip(self.batches, self.streams):
            s.wait_stream(cur)
            with torch.cuda.stream(s):
                b.apply(x_all, y_all, s)
        for s in self.streams[:len(self.batches)]:
            cur.wait_stream(s)

    def capture(self, x_all, y_all):
        """Record one apply on these buffers as a CUDA graph (replay with
        :meth:`replay`)."""
        import torch

        self.apply(x_all, y_all)  # warm-up outside capture
        torch.cuda.synchronize(self.dev)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.apply(x_all, y_all)
        self.graph = g
        return g

    def replay(self):
        self.graph.replay()

    def close(self):
        for b in self.batches:
            b.close()
