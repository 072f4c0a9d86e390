"""Serving form: many resident H-matrices, continuous batching of apply requests.

The reference serves one ``matmul`` call at a time and re-uploads the whole
representation on each (src/qhmat/cuda.cu:106-164).  Here:

* :class:`ServingPool` keeps matrices resident on one GPU under an HBM
  admission budget.  Uploads come from QHMAT001 images (the reference's file
  format, parsed and laid out once by ``qh_matrix_from_qhmat``); a new matrix
  is admitted when the budget allows, after evicting the least recently used
  idle matrices if needed, and refused (:class:`AdmissionError`) otherwise.
* :class:`ServingEngine` runs the request loop on a background thread.
  Requests name a resident matrix and a range of columns in that matrix's
  pinned host input buffer; results go to the same columns of its output
  buffer.  Requests that arrive while others are on the GPU wait only until a
  batch slot frees up: the loop takes every pending request of the matrix
  with the oldest waiting request (up to 64 columns), gathers their columns
  with one device kernel straight from pinned host memory, applies once (the
  precision form for two or more columns where the matrix's calibration chose
  it, else the plain FP64 form), scatters the result columns back, and
  records an event.  Several such batches are in flight at once on separate
  CUDA streams, so their work overlaps on the device.

Results do not depend on the mix: every column is computed with its own
fixed-point exponent, the precision form's scales are layout constants, and
the kernels accumulate each column independently, so a request gives the same
y alone and batched with others (tested).
"""

from __future__ import annotations

import collections
import ctypes as C
import itertools
import threading
import time
from dataclasses import dataclass, field

import numpy as np

from ._lib import load_library, raise_for
from .matrix import HMatrix, PrecisionHMatrix, qhmat_device_bytes


class AdmissionError(RuntimeError):
    """A matrix does not fit the HBM budget even after evicting idle ones."""


class AdmissionController:
    """Budget accounting for resident matrices (host logic only).

    ``reserve(key, nbytes)`` returns the keys to evict (least recently used
    first, never a pinned key) so that the new matrix fits, or raises
    :class:`AdmissionError`; ``commit`` records it; ``release`` frees it."""

    def __init__(self, budget_bytes: int):
        self.budget = int(budget_bytes)
        self.used = 0
        self._sizes: "collections.OrderedDict[object, int]" = collections.OrderedDict()
        self._pins: collections.Counter = collections.Counter()

    def __contains__(self, key) -> bool:
        return key in self._sizes

    def touch(self, key) -> None:
        self._sizes.move_to_end(key)

    def pin(self, key) -> None:
        self._pins[key] += 1

    def unpin(self, key) -> None:
        self._pins[key] -= 1
        if self._pins[key] <= 0:
            del self._pins[key]

    def reserve(self, key, nbytes: int) -> list:
        if key in self._sizes:
            raise ValueError(f"matrix {key!r} is already resident")
        if nbytes > self.budget:
            raise AdmissionError(f"matrix {key!r} needs {nbytes} bytes, more than the whole budget {self.budget}")
        free = self.budget - self.used
        victims = []
        for k, sz in self._sizes.items():
            if free >= nbytes:
                break
            if self._pins.get(k):
                continue
            victims.append(k)
            free += sz
        if free < nbytes:
            raise AdmissionError(f"matrix {key!r} needs {nbytes} bytes; {free} free after evicting every idle matrix")
        return victims

    def commit(self, key, nbytes: int) -> None:
        self._sizes[key] = int(nbytes)
        self.used += int(nbytes)

    def release(self, key) -> None:
        self.used -= self._sizes.pop(key)
        self._pins.pop(key, None)


@dataclass
class Resident:
    key: object
    plain: HMatrix
    pf: PrecisionHMatrix | None
    form: str
    device_bytes: int
    x_host: object = None  # pinned torch tensor (n, C) of inputs
    y_host: object = None  # pinned torch tensor (n, C) of outputs

    @property
    def order(self) -> int:
        return self.plain.order


class ServingPool:
    """Resident matrices on one device under an HBM budget (default 64 GiB)."""

    def __init__(self, device: int = 0, budget_bytes: int = 64 << 30, precision: bool = True):
        self.device = device
        self.precision = precision
        self.admission = AdmissionController(budget_bytes)
        self._res: dict = {}
        self._lock = threading.Lock()

    def admit(self, key, data: bytes, *, columns: int = 0) -> Resident:
        """Upload a QHMAT001 image; optionally attach pinned input/output
        buffers of ``columns`` columns for requests.  The image's device
        footprint is computed on the host first (the layouts the upload will
        build) and reserved -- evicting idle matrices if needed -- before any
        device allocation, so the budget holds throughout.  Raises
        AdmissionError (nothing becomes resident, nothing is evicted) if it
        cannot fit; a corrupt image raises before anything is reserved."""
        import torch

        sms = torch.cuda.get_device_properties(self.device).multi_processor_count
        plain_b, pf_b = qhmat_device_bytes(data, sms=sms, precision=self.precision)
        nbytes = plain_b + pf_b
        with self._lock:
            victims = self.admission.reserve(key, nbytes)
            for v in victims:
                self._drop(v)
            self.admission.commit(key, nbytes)
        plain = pf = None
        form = "plain"
        try:
            plain = HMatrix.from_bytes(data, device=self.device)
            if self.precision:
                pf = PrecisionHMatrix.from_bytes(data, device=self.device)
                form = plain.attach_precision(pf)["form"]
        except Exception:
            if pf is not None:
                pf.close()
            if plain is not None:
                plain.close()
            with self._lock:
                self.admission.release(key)
            raise
        actual = plain.stats["device_bytes"] + (pf.stats["device_bytes"] if pf is not None else 0)
        if actual != nbytes:  # the same layouts: equal by construction; keep the books exact regardless
            with self._lock:
                self.admission.release(key)
                self.admission.commit(key, actual)
            nbytes = actual
        r = Resident(key, plain, pf, form, nbytes)
        if columns:
            n = plain.order
            r.x_host = torch.zeros((n, columns), dtype=torch.float64).pin_memory()
            r.y_host = torch.zeros((n, columns), dtype=torch.float64).pin_memory()
        with self._lock:
            self._res[key] = r
        return r

    def _drop(self, key) -> None:
        r = self._res.pop(key, None)
        self.admission.release(key)
        if r is not None:
            if r.pf is not None:
                r.pf.close()
            r.plain.close()

    def evict(self, key) -> None:
        with self._lock:
            self._drop(key)

    def get(self, key) -> Resident:
        with self._lock:
            r = self._res[key]
            self.admission.touch(key)
            return r

    def keys(self) -> list:
        with self._lock:
            return list(self._res)

    @property
    def used_bytes(self) -> int:
        return self.admission.used


@dataclass
class Request:
    """Columns [col, col + k) of a resident matrix's input buffer."""
    rid: int
    key: object
    col: int
    k: int
    t_arrival: float
    t_done: float = 0.0
    done: bool = False
    cancelled: bool = False
    error: str = ""


@dataclass
class _Slot:
    stream: object
    event: object
    xbuf: object
    ybuf: object
    cols: object  # pinned int32 column list
    ws_plain: object = None
    ws_pf: object = None
    batch: list = field(default_factory=list)
    busy: bool = False


class ServingEngine:
    """Continuous-batching request loop over a :class:`ServingPool`.

    ``submit(key, col, k)`` enqueues a request (thread-safe) and returns it;
    ``request.done`` turns true, with ``t_done`` set, once its columns of the
    output buffer hold y.  ``cancel(request)`` drops a request that has not
    been dispatched yet.  Batches: up to ``max_cols`` columns of one matrix;
    ``streams`` x ``depth`` batches in flight; batches of plain-form
    matrices stop at ``plain_max_cols`` columns."""

    def __init__(self, pool: ServingPool, *, streams: int = 4, depth: int = 2, max_cols: int = 64,
                 plain_max_cols: int = 16, max_order: int = 1 << 15):
        import torch

        self.pool = pool
        self.max_cols = max_cols
        # the plain form's work grows with the columns it is given, so larger
        # batches only delay the requests behind them
        self.plain_max_cols = min(plain_max_cols, max_cols)
        self._lib = load_library()
        self._queue: collections.deque = collections.deque()
        self._pending: "collections.OrderedDict[object, collections.deque]" = collections.OrderedDict()
        self._lock = threading.Lock()
        self._ids = itertools.count()
        self._stop = threading.Event()
        self._thread = None
        dev = torch.device("cuda", pool.device)
        self._slots = []
        for _ in range(streams):
            st = torch.cuda.Stream(device=dev)
            for _ in range(depth):
                self._slots.append(_Slot(
                    stream=st, event=torch.cuda.Event(),
                    xbuf=torch.empty(max_order * max_cols, dtype=torch.float64, device=dev),
                    ybuf=torch.empty(max_order * max_cols, dtype=torch.float64, device=dev),
                    cols=torch.zeros(max_cols, dtype=torch.int32).pin_memory()))
        self.completed: list = []
        self.batches = 0
        self.batch_cols = 0

    # ------------------------------------------------------------ client side
    def submit(self, key, col: int, k: int, t_arrival: float | None = None) -> Request:
        """Enqueue columns [col, col + k) of matrix ``key``; ``t_arrival``
        (perf_counter seconds, default now) is the arrival the latency is
        measured from."""
        r = Request(next(self._ids), key, int(col), int(k),
                    time.perf_counter() if t_arrival is None else float(t_arrival))
        with self._lock:
            self._queue.append(r)
        return r

    def cancel(self, req: Request) -> bool:
        """Drop a request that has not been dispatched; True if it was dropped."""
        with self._lock:
            if req.done or req.cancelled:
                return False
            for q in [self._queue, *self._pending.values()]:
                if req in q:
                    q.remove(req)
                    req.cancelled = True
                    return True
        return False

    def start(self) -> "ServingEngine":
        self._thread = threading.Thread(target=self._loop, name="qhmat-serving", daemon=True)
        self._thread.start()
        return self

    def stop(self, drain: bool = True, timeout: float = 60.0) -> None:
        if drain:
            t0 = time.perf_counter()
            while time.perf_counter() - t0 < timeout:
                with self._lock:
                    idle = not self._queue and not any(self._pending.values())
                if idle and not any(s.busy for s in self._slots):
                    break
                time.sleep(0.001)
        self._stop.set()
        if self._thread is not None:
            self._thread.join(timeout=timeout)

    # ------------------------------------------------------------ the loop
    def _workspace(self, slot: _Slot, res: Resident, p: int, precision: bool):
        import torch

        need = res.pf.workspace_bytes(p) if precision else res.plain.workspace_bytes(p)
        attr = "ws_pf" if precision else "ws_plain"
        ws = getattr(slot, attr)
        if ws is None or ws.numel() < need:
            ws = torch.empty(need, dtype=torch.uint8, device=slot.xbuf.device)
            setattr(slot, attr, ws)
        return ws, need

    def _dispatch(self, slot: _Slot, key, batch: list) -> None:
        res = self.pool.get(key)
        n = res.order
        p = sum(r.k for r in batch)
        cols = slot.cols.numpy()
        j = 0
        for r in batch:
            cols[j:j + r.k] = np.arange(r.col, r.col + r.k, dtype=np.int32)
            j += r.k
        precision = res.form == "precision" and res.pf is not None and p >= 2
        ws, need = self._workspace(slot, res, p, precision)
        s = slot.stream.cuda_stream
        lib = self._lib
        C_in = res.x_host.shape[1]
        raise_for(lib.qh_gather_columns(res.x_host.data_ptr(), C_in, slot.xbuf.data_ptr(), p, slot.cols.data_ptr(),
                                        p, n, s))
        if precision:
            raise_for(lib.qh_pmatmul_device(res.pf._h, slot.xbuf.data_ptr(), slot.ybuf.data_ptr(), p,
                                            ws.data_ptr(), need, s, None))
        else:
            raise_for(lib.qh_matmul_device(res.plain._h, slot.xbuf.data_ptr(), slot.ybuf.data_ptr(), p,
                                           ws.data_ptr(), need, s, None))
        raise_for(lib.qh_scatter_columns(slot.ybuf.data_ptr(), p, res.y_host.data_ptr(), C_in, slot.cols.data_ptr(),
                                         p, n, s))
        slot.event.record(slot.stream)
        slot.batch = batch
        slot.busy = True
        self.pool.admission.pin(key)
        self.batches += 1
        self.batch_cols += p

    def _loop(self) -> None:
        while not self._stop.is_set():
            progressed = False
            with self._lock:
                while self._queue:
                    r = self._queue.popleft()
                    self._pending.setdefault(r.key, collections.deque()).append(r)
            # completions
            now = None
            for slot in self._slots:
                if slot.busy and slot.event.query():
                    now = now or time.perf_counter()
                    for r in slot.batch:
                        r.t_done = now
                        r.done = True
                    self.completed.extend(slot.batch)
                    self.pool.admission.unpin(slot.batch[0].key)
                    slot.batch = []
                    slot.busy = False
                    progressed = True
            # dispatch: oldest waiting request's matrix first
            for slot in self._slots:
                if slot.busy:
                    continue
                with self._lock:
                    live = [(q[0].t_arrival, key) for key, q in self._pending.items() if q]
                    if not live:
                        break
                    _, key = min(live)
                    q = self._pending[key]
                    res = self.pool.get(key)
                    cap = self.max_cols if res.form == "precision" else self.plain_max_cols
                    batch, cols = [], 0
                    while q and (not batch or cols + q[0].k <= cap):
                        r = q.popleft()
                        batch.append(r)
                        cols += r.k
                try:
                    self._dispatch(slot, key, batch)
                except Exception as exc:  # noqa: BLE001 - reported on the requests
                    for r in batch:
                        r.error = str(exc)
                        r.done = True
                        r.t_done = time.perf_counter()
                    self.completed.extend(batch)
                progressed = True
            if not progressed:
                time.sleep(20e-6)


def latency_summary(requests: list) -> dict:
    """p50 / p99 / mean latency (ms) of completed requests and their columns."""
    lat = np.array([r.t_done - r.t_arrival for r in requests if r.done and not r.error], np.float64) * 1e3
    if lat.size == 0:
        return {"requests": 0}
    return {"requests": int(lat.size), "p50_ms": float(np.percentile(lat, 50)),
            "p99_ms": float(np.percentile(lat, 99)), "mean_ms": float(lat.mean()),
            "rhs": int(sum(r.k for r in requests if r.done and not r.error))}
