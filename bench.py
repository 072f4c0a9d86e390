#!/usr/bin/env python3
"""Benchmark of the resident quantized H-matrix matvec (one JSON line).

Workload (default ``cfg2``): the plain method at scale -- n = 32768 points
uniform in the unit square (numpy default_rng(1)), kernel
A_ij = -log(|x_i - x_j| + 1e-3), leaf_size 64, bit widths (4,8,12,16,24,32),
single FP64 right-hand side drawn from the same generator after the points.
The requested tolerance 1e-8 is infeasible for this matrix in the reference
(InfeasibleError at block (0:64, 64:128)); 1e-7 and 3e-7 are infeasible at
n = 32768 too, so the matrix is built at the tightest feasible tolerance of
that ladder, 1e-6, and the line states both.  The matrix is constructed on
this machine by qhmat_gb300.construct (byte-identical to the reference's
from_dense + save on the same NumPy build); the data are synthetic.

A step is one apply y = A x.  ``value`` is the packed-byte traffic model
(codes + two FP64 scales per component + dense diagonal + x read + y write)
divided by the device time per step, with x and y resident in HBM; the
representation (~200 MB) is larger than the 129 MB L2, so no flush is needed
between steps.  ``e2e`` is the same metric through the host-buffer C-ABI call
(qh_matmul_host: x in from host memory, apply, y out to host memory, all
timed; on a coherent host link the kernels access the host buffers directly,
else pinned H2D and D2H copies).

``--impl reference`` times the reference's CPU HMatrix::matmul on the host
cores instead: the reference core compiled from its sources (oracle/_ref)
where that build loads, else the bit-identical plain-C restatement
(oracle/qhmat_oracle.c) with every host thread (and, for comparison, on one
thread, as the reference runs).  That process never loads the CUDA library.
Both arms print the same ``config``.

The line also states the result's error against the FP64 dense product A x
(evaluated from the points, outside the timed region) and samples the SM
clocks with nvidia-smi over a load window around the timed region.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOADS = {
    "cfg2": dict(n=32768, dim=2, seed=1, kernel="log", leaf=64, tol_requested=1e-8, tol=1e-6, rhs=1,
                 desc="plain at scale: n=32768 uniform unit square (seed 1), -log(r+1e-3), leaf 64, "
                      "widths 4/8/12/16/24/32, single RHS"),
    "cfg1": dict(n=2048, dim=1, seed=0, kernel="inverse", leaf=32, tol_requested=1e-6, tol=1e-6, rhs=4,
                 desc="plain CPU-runnable: n=2048 linspace, 1/(r+0.4), leaf 32, RHS 2048x4 seed 0"),
    "cfg3": dict(n=32768, dim=3, seed=2, kernel="yukawa", leaf=64, tol_requested=1e-6, tol=1e-6, rhs=64,
                 desc="precision form: n=32768 uniform unit cube (seed 2), exp(-r)/(r+0.05), leaf 64, "
                      "widths 4/8/12/16/24/32, X 32768x64 N(0,1)"),
}
PRECISION_WORKLOADS = {"cfg3"}
SERVING_WORKLOADS = {"cfg5"}
BATCHING_WORKLOADS = {"cfg4"}
WORKLOADS["cfg4"] = dict(n=8192, dim=0, seed=3, kernel="mixed", leaf=0, tol_requested=0.0, tol=0.0, rhs=32,
                         desc="batching: 256 matrices, n log-uniform in [512, 8192], 1-D or 2-D uniform points, "
                              "1/(r+0.4) or -log(r+1e-3), tolerance log-uniform in [1e-8, 1e-4] escalated x10^0.25 "
                              "until feasible, leaf 16/32/64, 1-32 N(0,1) columns each (seed 3)")
WORKLOADS["cfg5"] = dict(n=32768, dim=0, seed=4, kernel="mixed", leaf=0, tol_requested=0.0, tol=0.0, rhs=16,
                         desc="serving: 16 resident matrices (4 each of n=1024/4096/16384/32768, 1-D or 2-D uniform "
                              "points, 1/(r+0.4) or -log(r+1e-3), tolerance log-uniform in [1e-8, 1e-4] escalated "
                              "x10^0.25 until feasible, leaf 16/32/64; seed 4), uploads at 1/s under a 64 GB budget, "
                              "Poisson arrivals at 20k requests/s of 1-16 N(0,1) columns")


def matrix_specs(count: int, seed: int, n_values=None) -> list:
    """Seeded matrix specs of the batched and served workloads: n log-uniform
    in [512, 8192] (or cycling through ``n_values``), 1-D or 2-D uniform
    points, kernel 1/(r+0.4) or -log(r+1e-3), tolerance log-uniform in
    [1e-8, 1e-4], leaf 16/32/64, 1..32 right-hand-side columns."""
    import math

    import numpy as np

    rng = np.random.default_rng(seed)
    specs = []
    for i in range(count):
        n = int(round(math.exp(rng.uniform(math.log(512), math.log(8192)))))
        if n_values is not None:
            n = int(n_values[i % len(n_values)])
        dim = int(rng.integers(1, 3))
        kernel = "inverse" if rng.integers(0, 2) == 0 else "log"
        tol = float(math.exp(rng.uniform(math.log(1e-8), math.log(1e-4))))
        leaf = int(rng.choice([16, 32, 64]))
        rhs = int(rng.integers(1, 33))
        specs.append(dict(n=n, dim=dim, kernel=kernel, tol=tol, leaf=leaf, rhs=rhs, seed=int(rng.integers(1 << 31))))
    return specs


def build_spec(spec: dict, workers: int, checksum=None, svd: str = "exact"):
    """(QHMAT001 image, effective tolerance, attempts) of one spec, with the
    deterministic escalation rule (x10^0.25 per InfeasibleError)."""
    import numpy as np

    from qhmat_gb300 import construct

    pts = np.random.default_rng(spec["seed"]).random((spec["n"], spec["dim"]))
    img, tol, attempts = construct.from_kernel_escalating(pts, spec["kernel"], tolerance=spec["tol"],
                                                          leaf_size=spec["leaf"], workers=workers, svd=svd)
    return construct.to_qhmat_bytes(img, checksum=checksum), tol, attempts


def _build_spec_job(args):
    spec, svd = args
    return build_spec(spec, 1, svd=svd)


def build_specs(specs: list, workers: int, svd: str = "exact") -> list:
    """Build many specs: small matrices one per worker process (spawn pool),
    large ones block-parallel; results in spec order."""
    import multiprocessing as mp

    small = [i for i, sp in enumerate(specs) if sp["n"] <= 8192]
    large = [i for i, sp in enumerate(specs) if sp["n"] > 8192]
    out = [None] * len(specs)
    if small:
        env = {k: os.environ.get(k) for k in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS")}
        for k in env:
            os.environ[k] = "1"
        try:
            with mp.get_context("spawn").Pool(max(1, workers)) as pool:
                for i, res in zip(small, pool.imap(_build_spec_job, [(specs[i], svd) for i in small])):
                    out[i] = res
        finally:
            for k, v in env.items():
                if v is None:
                    os.environ.pop(k, None)
                else:
                    os.environ[k] = v
    for i in large:
        out[i] = build_spec(specs[i], workers, svd=svd)
    return out


def make_inputs(name: str, workers: int, checksum=None, with_points: bool = False):
    """(QHMAT001 image, x, construction seconds[, points]) of a workload.

    ``checksum`` computes the image's trailer (default: the library's FNV-1a)."""
    import numpy as np

    from qhmat_gb300 import construct

    wl = WORKLOADS[name]
    if name == "cfg1":
        pts = np.linspace(0, 1, wl["n"])[:, None]
        x = np.random.default_rng(0).standard_normal((wl["n"], wl["rhs"]))
    else:
        rng = np.random.default_rng(wl["seed"])
        pts = rng.random((wl["n"], wl["dim"]))
        x = rng.standard_normal(wl["n"]) if wl["rhs"] == 1 else rng.standard_normal((wl["n"], wl["rhs"]))
    t0 = time.time()
    img = construct.from_kernel(pts, wl["kernel"], tolerance=wl["tol"], leaf_size=wl["leaf"],
                                workers=workers)
    data = construct.to_qhmat_bytes(img, checksum=checksum)
    if with_points:
        return data, x, time.time() - t0, pts
    return data, x, time.time() - t0


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, one sample every 200 ms, read by a
    background thread.  ``wait_first()`` blocks until the first sample has
    arrived (nvidia-smi takes a moment to start), so that the load window
    around the timed region is covered."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []
        self.error = ""
        self._thread = None

    def __enter__(self):
        import shutil
        import threading

        exe = shutil.which("nvidia-smi")
        if exe is None:
            self.error = "nvidia-smi not found on PATH"
            return self
        try:
            self.proc = subprocess.Popen(
                [exe, f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-i", str(self.index), "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
        except OSError as exc:
            self.error = f"nvidia-smi failed to start: {exc}"
            return self

        def reader():
            for ln in self.proc.stdout:
                if ln.strip():
                    self.lines.append(ln.strip())

        self._thread = threading.Thread(target=reader, daemon=True)
        self._thread.start()
        return self

    def wait_first(self, timeout: float = 10.0) -> bool:
        t0 = time.time()
        while self.proc is not None and not self.lines and time.time() - t0 < timeout:
            if self.proc.poll() is not None:
                break
            time.sleep(0.02)
        return bool(self.lines)

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                _, err = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                _, err = self.proc.communicate()
            if self._thread is not None:
                self._thread.join(timeout=5)
            if not self.lines and err:
                self.error = "nvidia-smi: " + err.strip().splitlines()[-1][:200]

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            f = [v.strip() for v in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0,
                    "note": self.error or "no samples"}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm),
                "window": "every 200 ms while the GPU ran untimed applies, the timed applies, "
                          "and untimed applies again (>= 1 s of load around the timed region)"}


def measured_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs, burst copy)"
    return 6800.0, "fallback (6.8 TB/s)"


def cpu_baseline(data: bytes, x, model_bytes: int, budget_s: float = 10.0) -> tuple[dict, object]:
    """The reference's CPU apply on the host cores over a bounded sample.

    The reference core compiled from its sources (oracle/_ref) where that
    build loads on this machine (it is single-threaded, as written), else the
    bit-identical C restatement (oracle/qhmat_oracle.c) on every host thread,
    plus a single-thread run of the same for comparison with the reference's
    own threading."""
    from oracle import oracle

    threads = os.cpu_count() or 1
    kind, impl = "port", None
    if oracle.reference_available():
        try:
            impl = oracle.RefMatrix(data)
            kind, threads = "reference", 1
        except OSError:
            impl = None
    if impl is None:
        impl = oracle.OracleMatrix(data)

    def timed(fn, budget):
        y = fn()  # warm-up
        reps, t0 = 0, time.perf_counter()
        while reps < 3 or (time.perf_counter() - t0 < budget and reps < 10000):
            fn()
            reps += 1
        return y, reps, time.perf_counter() - t0

    if kind == "reference":
        y, reps, dt = timed(lambda: impl.matmul(x), budget_s)
    else:
        y, reps, dt = timed(lambda: impl.matmul(x, threads=threads), budget_s)
    out = {"value": model_bytes * reps / dt / 1e9, "unit": "GB/s", "cores": threads, "kind": kind,
           "sample": f"{reps} full applies of the bench workload in {dt:.1f} s "
                     f"({1e3 * dt / reps:.2f} ms each, {threads} thread(s))",
           "ms_per_apply": 1e3 * dt / reps}
    if kind == "port" and threads > 1:
        _, r1, d1 = timed(lambda: impl.matmul(x, threads=1), min(budget_s, 5.0))
        out["single_thread"] = {"value": model_bytes * r1 / d1 / 1e9, "unit": "GB/s", "cores": 1,
                                "ms_per_apply": 1e3 * d1 / r1,
                                "note": "the same port on one thread (the reference's matmul is "
                                        "single-threaded)"}
    if kind == "port":
        out["why_port"] = ("the reference core is compiled from its own sources where they lie; "
                           "they are not on this machine, and no copy of them travels with the repo")
    return out, y


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(value: float, pg=None, device=None) -> float:
    """The largest of every rank's value (the whole job ends with its slowest
    replica); the value itself on one rank."""
    if pg is None:
        return float(value)
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def whole_job_gbs(model_bytes: int, world: int, ms_per_step: float) -> float:
    """Whole-job throughput of `world` replicas, each moving `model_bytes` per
    step, over the slowest replica's time per step."""
    return model_bytes * world / (ms_per_step * 1e-3) / 1e9


def run_reference_arm(args):
    """The reference's CPU apply on the bench workload (rank 0 only).  This
    process never loads the CUDA library: the image's trailer is computed by
    the C restatement, and the model bytes are read from the image."""
    world, rank, _ = dist_setup()
    if rank != 0:
        return 0
    from oracle import oracle

    data, x, build_s = make_inputs(args.workload, os.cpu_count() or 1, checksum=oracle.fnv1a64)
    wl = WORKLOADS[args.workload]
    model = _model_bytes(data, x)
    base, _ = cpu_baseline(data, x, model, budget_s=min(30.0, 5.0 + 0.02 * args.steps))
    out = {
        "impl": "reference", "metric": METRIC, "value": base["value"], "unit": "GB/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": model / (base["value"] * 1e9) * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": DATA_NOTE,
        "config": _config(args.workload, wl), "construction_s": round(build_s, 1),
        "cpu_baseline": base,
        "e2e": {"value": base["value"], "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)
    return 0


def _model_bytes(data: bytes, x) -> int:
    """Packed-byte model from a QHMAT001 image (read by the C restatement; no
    device needed)."""
    from oracle import oracle

    m = oracle.OracleMatrix(data)
    codes = scales = dense = 0
    for b in range(m.block_count):
        info = m.block_info(b)
        if info["dense"]:
            dense += 8 * (info["row1"] - info["row0"]) * (info["col1"] - info["col0"])
        else:
            codes += 4 * (info["left_words"] + info["right_words"])
            scales += 16 * info["rank"]
    rhs = 1 if x.ndim == 1 else x.shape[1]
    return codes + scales + dense + 16 * m.order * rhs


METRIC = "H-matvec GB/s (% HBM peak)"
DATA_NOTE = "synthetic (seeded points; matrix constructed on the host)"


def _config(name, wl):
    """The workload description, identical in both arms."""
    return {"workload": f"{name}: {wl['desc']}", "n": wl["n"], "rhs": wl["rhs"],
            "tolerance": wl["tol"], "tolerance_requested": wl["tol_requested"],
            "tolerance_note": ("requested tolerance infeasible in the reference; tightest feasible of "
                               "the ladder 1e-8/3e-8/1e-7/3e-7/1e-6") if wl["tol"] != wl["tol_requested"] else "",
            "l2": "representation larger than L2 (129 MB; 1.3 GB for the precision workload); no flush between steps"}


def dense_oracle_error(pts, kernel: str, x, y, device) -> dict:
    """||y - A x|| / ||A x|| with A x the FP64 dense product, evaluated on the GPU
    in row chunks from the points (A itself is never formed); outside any
    timed region."""
    import numpy as np
    import torch

    P = torch.from_numpy(np.ascontiguousarray(pts, dtype=np.float64)).to(device)
    X = torch.from_numpy(np.ascontiguousarray(x, dtype=np.float64)).to(device)
    if X.ndim == 1:
        X = X[:, None]
    out = torch.empty_like(X)
    for r0 in range(0, P.shape[0], 1024):
        r = torch.cdist(P[r0:r0 + 1024], P, compute_mode="donot_use_mm_for_euclid_dist")
        if kernel == "log":
            a = -torch.log(r + 1e-3)
        elif kernel == "inverse":
            a = 1.0 / (r + 0.4)
        else:
            a = torch.exp(-r) / (r + 0.05)
        out[r0:r0 + 1024] = a @ X
    ax = out.cpu().numpy().reshape(np.shape(y))
    return {"rel_err_vs_dense_Ax": float(np.linalg.norm(y - ax) / np.linalg.norm(ax)),
            "oracle": "FP64 dense A x from the points (GPU, row chunks of 1024; A never stored)"}


def run_precision(args):
    """The multi-right-hand-side precision form on its workload (X 32768 x 64):
    RHS/s of the tcgen05 apply (device buffers, CUDA events), beside the plain
    FP64 form on the same X, the error of both against the dense product, the
    gate between them, and the tensor / HBM rooflines of the dominant kernel."""
    import ctypes as C

    import numpy as np

    world, rank, local = dist_setup()
    workers = max(1, (os.cpu_count() or 1) // max(1, world))
    data, x, build_s, pts = make_inputs(args.workload, workers, with_points=True)

    import torch

    import qhmat_gb300
    from qhmat_gb300 import _lib, precision_gate

    torch.cuda.set_device(local)
    pg = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
        pg = dist
    lib = _lib.load_library()
    wl = WORKLOADS[args.workload]
    rhs = wl["rhs"]
    h = qhmat_gb300.HMatrix.from_bytes(data, device=local, precision=True)
    pf = h._pf
    pst = pf.stats
    dev = torch.device("cuda", local)
    xd = torch.from_numpy(np.ascontiguousarray(x)).to(dev)
    yd = torch.empty_like(xd)
    need = pf.workspace_bytes(rhs)
    ws = torch.empty(need, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)

    def step():
        rc = lib.qh_pmatmul_device(pf._h, xd.data_ptr(), yd.data_ptr(), rhs, ws.data_ptr(), need,
                                   stream.cuda_stream, None)
        if rc:
            _lib.raise_for(rc)

    # per-kernel breakdown (separate pass, events between the launches)
    KP = min(args.steps, 20)
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(5)] for _ in range(KP)]
    for row in evs:
        for e in row:
            e.record(stream)
    torch.cuda.synchronize()
    for i in range(KP):
        arr = (C.c_void_p * 5)(*[e.cuda_event for e in evs[i]])
        _lib.raise_for(lib.qh_pmatmul_device_profiled(pf._h, xd.data_ptr(), yd.data_ptr(), rhs, ws.data_ptr(), need,
                                                      stream.cuda_stream, None, arr))
    torch.cuda.synchronize()
    names = ["prep", "column", "row", "combine"]
    kmean = {k: statistics.mean(evs[i][j].elapsed_time(evs[i][j + 1]) for i in range(KP))
             for j, k in enumerate(names)}
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    K = args.steps
    t0e, t1e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        clk.wait_first()
        t_load = time.perf_counter()
        while time.perf_counter() - t_load < 0.6:
            step()
            torch.cuda.synchronize()
        if pg:
            pg.barrier()
        torch.cuda.synchronize()
        t0e.record(stream)
        for _ in range(K):
            step()
        t1e.record(stream)
        torch.cuda.synchronize()
        if pg:
            pg.barrier()
        t_load = time.perf_counter()
        while time.perf_counter() - t_load < 0.4:
            step()
            torch.cuda.synchronize()
    ms_step = max_over_ranks(t0e.elapsed_time(t1e), pg, dev) / K
    y_pf = yd.cpu().numpy()

    # the plain FP64 form on the same X (device buffers; one chain per apply)
    nplain = 3
    ws_plain = torch.empty(h.workspace_bytes(rhs), dtype=torch.uint8, device=dev)
    yp = torch.empty_like(xd)

    def plain_step():
        _lib.raise_for(lib.qh_matmul_device(h._h, xd.data_ptr(), yp.data_ptr(), rhs, ws_plain.data_ptr(),
                                            ws_plain.numel(), stream.cuda_stream, None))

    plain_step()
    torch.cuda.synchronize()
    p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    p0.record(stream)
    for _ in range(nplain):
        plain_step()
    p1.record(stream)
    torch.cuda.synchronize()
    ms_plain = p0.elapsed_time(p1) / nplain
    y_plain = yp.cpu().numpy()

    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    tc_peak = float(peaks.get("bf16_tflops", 1900.0))
    N = 3 * min(rhs, 64)
    n = h.order
    nslot = pst["row_slots"]
    pu = (min(rhs, 64) + 15) // 16 * 16
    # per kernel: MMA flops issued (f16, N = 3p limb columns) and the bytes it
    # must move (digit planes / limb tiles, u per slot, x limbs, partials)
    kflops = {"column": 2.0 * pst["mma_col_elements"] * N, "row": 2.0 * pst["mma_row_elements"] * N}
    kbytes = {"column": pst["stored_q_bytes"] + 4 * nslot * pu + 2 * N * n,
              "row": pst["stored_p_bytes"] + pst["stored_dense_bytes"] + 4 * nslot * pu + 8 * n * pu}
    dom = max(("column", "row"), key=lambda k: kmean[k])
    tfrac = kflops[dom] / (kmean[dom] * 1e-3) / 1e12 / tc_peak
    hfrac = kbytes[dom] / (kmean[dom] * 1e-3) / 1e9 / hbm_peak
    bound = "tensor" if tfrac >= hfrac else "hbm"
    achieved = (kflops[dom] / (kmean[dom] * 1e-3) / 1e12) if bound == "tensor" else \
        (kbytes[dom] / (kmean[dom] * 1e-3) / 1e9)
    model_bytes = h.model_bytes(rhs)
    model_flops = rhs * h.stats["flops_per_rhs"]
    value = rhs * world / (ms_step * 1e-3)
    traffic = None
    traffic_file = ROOT / "profiles" / f"traffic_{args.workload}.json"
    if traffic_file.exists():
        try:
            traffic = json.loads(traffic_file.read_text()).get(dom)
        except ValueError:
            traffic = None
    out = {
        "metric": "H-matvec RHS/s (precision form, X 32768x64)", "value": round(value, 1), "unit": "RHS/s",
        "n_gpus": world, "steps": K, "warmup": args.warmup, "ms_per_step": round(ms_step, 5),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f16 digit planes x f16 hi/mid/lo limbs of x and u, f32 accumulate (tcgen05, TMEM); "
                 "f64 scales, dense-limb sums and y",
        "data": DATA_NOTE, "config": _config(args.workload, wl), "construction_s": round(build_s, 1),
        "roofline": {"bound": bound, "kernel": dom, "achieved": round(achieved, 1),
                     "peak": tc_peak if bound == "tensor" else hbm_peak,
                     "unit": "TFLOP/s" if bound == "tensor" else "GB/s",
                     "frac": round(max(tfrac, hfrac), 4), "traffic": traffic,
                     "tensor_frac": round(tfrac, 4), "hbm_frac": round(hfrac, 4),
                     "kernel_ms": {k: round(v, 5) for k, v in kmean.items()},
                     "mma_flops": kflops, "moved_bytes": kbytes,
                     "peak_source": "MEASURED_PEAKS.json (bf16_tflops burst; f16 runs at the bf16 rate; hbm_gbs)"},
        "model": {"packed_bytes": model_bytes, "flops": model_flops,
                  "packed_gbs": round(model_bytes / (ms_step * 1e-3) / 1e9, 1)},
        "plain_form": {"ms_per_apply": round(ms_plain, 4), "rhs_per_s": round(rhs / (ms_plain * 1e-3), 1),
                       "speedup_of_precision_form": round(ms_plain / ms_step, 2)},
        "gpu_launches": int(pst["launches_per_pass"]) * ((rhs + 63) // 64) * K,
        "clocks": clk.summary(),
        "stats": pst,
    }
    if rank == 0:
        gate = precision_gate(y_pf, y_plain, x, h.reconstruction_bound)
        acc_pf = dense_oracle_error(pts, wl["kernel"], x, y_pf, dev)
        acc_plain = dense_oracle_error(pts, wl["kernel"], x, y_plain, dev)
        out["accuracy"] = {
            "precision_rel_err_vs_dense_Ax": acc_pf["rel_err_vs_dense_Ax"],
            "plain_rel_err_vs_dense_Ax": acc_plain["rel_err_vs_dense_Ax"],
            "gate": "per column max|y_pf - y_plain| <= 0.01 * reconstruction_bound * ||x||_1",
            "gate_worst_ratio": gate["worst_ratio"], "gate_passes": gate["passes"],
            "max_abs_dev_vs_plain": gate["max_abs_dev"], "rel_dev_vs_plain": gate["rel_err"],
            "raw_0.01_bound": 0.01 * h.reconstruction_bound,
            "reconstruction_bound": h.reconstruction_bound,
            "calibration": h.form_choice,
        }
        # e2e: NumPy X in, Y out (H2D and D2H copies inside the timed region)
        xh = np.ascontiguousarray(x)
        pf.matmul(xh)
        t0 = time.perf_counter()
        ne = max(3, min(args.e2e_steps, 20))
        for _ in range(ne):
            yh = pf.matmul(xh)
        e2e = (time.perf_counter() - t0) / ne
        out["e2e"] = {"value": round(rhs / e2e, 1), "unit": "RHS/s", "h2d_bytes_per_step": int(xh.nbytes),
                      "d2h_bytes_per_step": int(yh.nbytes), "ms_per_step": round(1e3 * e2e, 4),
                      "transfer": ("qh_pmatmul_host: X read and Y written by the kernels in the caller's NumPy "
                                   "buffers over the coherent host link" if pf.host_direct else
                                   "qh_pmatmul_host: pinned staging, one H2D copy of X and one D2H copy of Y")}
        if not args.no_cpu_baseline:
            from oracle import oracle

            om = oracle.OracleMatrix(data)
            threads = os.cpu_count() or 1
            xs = np.ascontiguousarray(x[:, :2])
            om.matmul(xs[:, :1], threads=threads)
            t0 = time.perf_counter()
            reps = 0
            while reps < 1 or time.perf_counter() - t0 < 10.0:
                om.matmul(xs, threads=threads)
                reps += 1
            dt = time.perf_counter() - t0
            out["cpu_baseline"] = {"value": round(2 * reps / dt, 3), "unit": "RHS/s", "cores": threads,
                                   "kind": "port",
                                   "sample": f"{reps} applies of 2 of the 64 columns in {dt:.1f} s ({threads} threads)"}
        print(json.dumps(out), flush=True)
    if pg:
        pg.barrier()
        pg.destroy_process_group()
    return 0


def run_batching(args):
    """The batching form: 256 matrices applied as one CUDA graph launch
    (block-diagonal persistent kernels, per-matrix form choice, autotuned
    precision schedule) against one plain launch chain per matrix."""
    world, rank, local = dist_setup()
    if rank != 0:
        return 0
    import ctypes as C

    import numpy as np

    t0 = time.time()
    specs = matrix_specs(256, 3)
    built = build_specs(specs, os.cpu_count() or 1, svd="randomized")
    build_s = time.time() - t0
    images = [b[0] for b in built]
    rhs = [sp["rhs"] for sp in specs]

    import torch

    from qhmat_gb300 import HMatrix, _lib, precision_gate
    from qhmat_gb300.batching import BatchedHMatrices

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    t1 = time.time()
    bat = BatchedHMatrices(images, rhs, device=local, forms="auto", autotune=True,
                           cache=os.environ.get("QHMAT_GB300_AUTOTUNE", "/tmp/qhmat_gb300_autotune.json"))
    setup_s = time.time() - t1
    rng = np.random.default_rng(3)
    xh_in = rng.standard_normal(bat.total)
    x_all = torch.from_numpy(xh_in).to(dev)
    y_all = torch.zeros_like(x_all)
    bat.capture(x_all, y_all)
    s = torch.cuda.current_stream(dev)
    K, W = args.steps, args.warmup
    for _ in range(W):
        bat.replay()
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        clk.wait_first()
        tl = time.perf_counter()
        while time.perf_counter() - tl < 0.5:
            bat.replay()
            torch.cuda.synchronize(dev)
        e0.record(s)
        for _ in range(K):
            bat.replay()
        e1.record(s)
        torch.cuda.synchronize(dev)
    ms_batch = e0.elapsed_time(e1) / K
    y_batch = y_all.cpu().numpy()

    # end to end: the packed X copied in from pinned host memory, one graph
    # launch, the packed Y copied back, every step
    x_pin = torch.from_numpy(rng.standard_normal(bat.total)).pin_memory()
    y_pin = torch.empty_like(x_pin).pin_memory()
    ne = max(3, K // 2)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for _ in range(ne):
        x_all.copy_(x_pin, non_blocking=True)
        bat.replay()
        y_pin.copy_(y_all, non_blocking=True)
        torch.cuda.synchronize(dev)
    ms_e2e = (time.perf_counter() - t0) / ne * 1e3
    x_all.copy_(torch.from_numpy(np.ascontiguousarray(xh_in)))
    bat.replay()
    torch.cuda.synchronize(dev)

    # baseline: one plain launch chain per matrix, eager, on one stream
    lib = _lib.load_library()
    hs = [HMatrix.from_bytes(img, device=local) for img in images]
    y_plain = torch.zeros_like(x_all)
    wss = [torch.empty(max(h.workspace_bytes(r), 256), dtype=torch.uint8, device=dev) for h, r in zip(hs, rhs)]
    offs = [int(v) for v in bat.x_offsets]

    def per_matrix():
        for k, h in enumerate(hs):
            xp = x_all.data_ptr() + 8 * offs[k]
            yp = y_plain.data_ptr() + 8 * offs[k]
            _lib.raise_for(lib.qh_matmul_device(h._h, xp, yp, rhs[k], wss[k].data_ptr(), wss[k].numel(),
                                                s.cuda_stream, None))

    per_matrix()
    torch.cuda.synchronize(dev)
    b0, b1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    nb = max(3, K // 4)
    b0.record(s)
    for _ in range(nb):
        per_matrix()
    b1.record(s)
    torch.cuda.synchronize(dev)
    ms_plain = b0.elapsed_time(b1) / nb
    yp_h = y_plain.cpu().numpy()
    xh = x_all.cpu().numpy()
    worst, plain_bitwise = 0.0, True
    for k in range(len(images)):
        a, b = offs[k], offs[k + 1]
        shape = (bat.orders[k], rhs[k])
        if bat.form[k] == "plain":
            plain_bitwise &= bool(np.array_equal(y_batch[a:b], yp_h[a:b]))
        else:
            g = precision_gate(y_batch[a:b].reshape(shape), yp_h[a:b].reshape(shape), xh[a:b].reshape(shape),
                               bat.bounds[k])
            worst = max(worst, g["worst_ratio"])
    total_rhs = int(sum(rhs))
    out = {
        "metric": "batched H-matvec RHS/s (256 matrices, one graph launch)",
        "value": round(total_rhs / (ms_batch * 1e-3), 1), "unit": "RHS/s", "n_gpus": 1, "steps": K, "warmup": W,
        "ms_per_step": round(ms_batch, 4), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "per matrix: f64 plain form or f16-limb precision form (calibrated)",
        "data": "synthetic (seeded points and right-hand sides; matrices constructed on the host)",
        "config": {"workload": f"cfg4: {WORKLOADS['cfg4']['desc']}", "construction_s": round(build_s, 1),
                   "construction": "randomized SVD for blocks wider than 128 (seeded; same residual checks)",
                   "effective_tolerances": [b[1] for b in built], "escalations": [b[2] for b in built]},
        "forms": {"precision": bat.form.count("precision"), "plain": bat.form.count("plain")},
        "autotune": bat.tuning, "setup_s": round(setup_s, 1),
        "per_matrix_plain": {"ms_per_batch": round(ms_plain, 4), "rhs_per_s": round(total_rhs / (ms_plain * 1e-3), 1),
                             "launches": 4 * len(images)},
        "speedup_vs_per_matrix_plain": round(ms_plain / ms_batch, 2),
        "parity": {"plain_matrices_bitwise_equal_to_own_apply": plain_bitwise,
                   "precision_matrices_worst_gate_ratio": worst},
        "gpu_launches": "one CUDA graph per step",
        "clocks": clk.summary(),
        "e2e": {"value": round(total_rhs / (ms_e2e * 1e-3), 1), "unit": "RHS/s",
                "h2d_bytes_per_step": int(x_pin.numel() * 8), "d2h_bytes_per_step": int(y_pin.numel() * 8),
                "ms_per_step": round(ms_e2e, 4),
                "transfer": "packed X copied in from pinned host memory, one graph launch, packed Y copied back"},
        "precision_segment_chunks": bat.pf_seg,
    }
    print(json.dumps(out), flush=True)
    for h in hs:
        h.close()
    bat.close()
    return 0


def run_serving(args):
    """The serving form under Poisson load (rank 0; the other ranks exit):
    RHS/s served and p50/p99 request latency of the continuous-batching loop,
    beside the plain per-request kernel on the same arrival schedule."""
    world, rank, local = dist_setup()
    if rank != 0:
        return 0
    import numpy as np

    t0 = time.time()
    workers = os.cpu_count() or 1
    specs = matrix_specs(16, 4, n_values=(1024, 4096, 16384, 32768))
    uploads = matrix_specs(4, 40, n_values=(1024, 4096))
    built = build_specs(specs + uploads, workers, svd="randomized")
    build_s = time.time() - t0

    import torch

    from qhmat_gb300 import precision_gate
    from qhmat_gb300.serving import ServingEngine, ServingPool, latency_summary

    torch.cuda.set_device(local)
    C_cols = 256
    pool = ServingPool(device=local, budget_bytes=64 << 30)
    rng = np.random.default_rng(4)
    keys = []
    for i, (data, tol, att) in enumerate(built[:16]):
        r = pool.admit(f"m{i}", data, columns=C_cols)
        r.x_host.copy_(torch.from_numpy(rng.standard_normal((r.order, C_cols))))
        keys.append(f"m{i}")
    forms = {k: pool.get(k).form for k in keys}
    T = float(os.environ.get("QHMAT_GB300_SERVE_SECONDS", "2.0"))
    sys.setswitchinterval(2e-4)  # the serving thread and the load generator share the interpreter
    engine = ServingEngine(pool, streams=6, depth=2, max_cols=64, plain_max_cols=16, max_order=32768).start()
    dev = torch.device("cuda", local)
    from qhmat_gb300 import _lib as L

    lib = L.load_library()
    xb = torch.empty(32768 * 16, dtype=torch.float64, device=dev)
    yb = torch.empty_like(xb)
    colsb = torch.zeros(16, dtype=torch.int32).pin_memory()
    wsb = {}

    def schedule(rate, seed):
        g = np.random.default_rng(seed)
        n_req = int(rate * T * 1.2) + 16
        times = np.cumsum(g.exponential(1.0 / rate, n_req))
        times = times[times < T]
        return times, g.integers(0, len(keys), times.size), g.integers(1, 17, times.size)

    def col_alloc():
        ring = {k: 0 for k in keys}

        def col_for(key, k):
            c = ring[key]
            if c + k > C_cols:
                c = 0
            ring[key] = c + k
            return c
        return col_for

    def served_phase(rate, seed):
        times, req_keys, req_k = schedule(rate, seed)
        col_for = col_alloc()
        reqs = []
        b0, bt0 = engine.batches, engine.batch_cols
        start = time.perf_counter()
        i, n = 0, times.size
        while i < n:
            # submit every request whose arrival time has come, stamped with
            # its scheduled arrival; sleep (releasing the interpreter lock to
            # the serving thread) until the next one
            now = time.perf_counter() - start
            while i < n and times[i] <= now:
                key = keys[int(req_keys[i])]
                k = int(req_k[i])
                reqs.append(engine.submit(key, col_for(key, k), k, t_arrival=start + float(times[i])))
                i += 1
            if i < n:
                time.sleep(max(0.0, min(1e-4, times[i] - (time.perf_counter() - start))))
        t_wait = time.perf_counter()
        while not all(r.done for r in reqs) and time.perf_counter() - t_wait < 120:
            time.sleep(0.001)
        lat = latency_summary(reqs)
        wall = max(r.t_done for r in reqs) - start
        nb = engine.batches - b0
        return reqs, {"offered_requests_per_s": rate, "requests": len(reqs), **lat,
                      "rhs_per_s": round(lat.get("rhs", 0) / wall, 1), "wall_s": round(wall, 3),
                      "batches": nb, "mean_batch_columns": round((engine.batch_cols - bt0) / max(1, nb), 2)}

    def plain_phase(rate, seed, max_wall):
        """One plain apply per request, in arrival order, on one stream, for
        at most ``max_wall`` seconds (later requests are not served)."""
        times, req_keys, req_k = schedule(rate, seed)
        col_for = col_alloc()
        st = torch.cuda.current_stream(dev)
        lat, rhs_done = [], 0
        n = times.size
        start = time.perf_counter()
        for i in range(times.size):
            if time.perf_counter() - start > max_wall:
                n = i
                break
            t_arr, key, k = times[i], keys[int(req_keys[i])], int(req_k[i])
            while time.perf_counter() - start < t_arr:
                pass
            r = pool.get(key)
            c0 = col_for(key, k)
            colsb.numpy()[:k] = np.arange(c0, c0 + k, dtype=np.int32)
            need = r.plain.workspace_bytes(k)
            if wsb.get(key) is None or wsb[key].numel() < need:
                wsb[key] = torch.empty(max(need, 1), dtype=torch.uint8, device=dev)
            L.raise_for(lib.qh_gather_columns(r.x_host.data_ptr(), C_cols, xb.data_ptr(), k, colsb.data_ptr(), k,
                                              r.order, st.cuda_stream))
            L.raise_for(lib.qh_matmul_device(r.plain._h, xb.data_ptr(), yb.data_ptr(), k, wsb[key].data_ptr(), need,
                                             st.cuda_stream, None))
            torch.cuda.synchronize(dev)
            lat.append(time.perf_counter() - start - t_arr)
            rhs_done += k
        wall = time.perf_counter() - start
        ll = np.array(lat) * 1e3
        return {"offered_requests_per_s": rate, "requests_offered": int(times.size), "requests_served": n,
                "p50_ms": float(np.percentile(ll, 50)), "p99_ms": float(np.percentile(ll, 99)),
                "rhs_per_s": round(rhs_done / wall, 1),
                "note": f"one plain apply per request in arrival order; {n} of {times.size} served within "
                        f"{max_wall:.0f} s (latencies of the unserved ones would be larger still)"}

    stop_uploads = threading.Event()
    upload_log = []

    def uploader():
        for j, (data, tol, att) in enumerate(built[16:]):
            if stop_uploads.wait(1.0):
                return
            t = time.perf_counter()
            try:
                pool.admit(f"up{j}", data, columns=C_cols)
                upload_log.append({"key": f"up{j}", "s": round(time.perf_counter() - t, 3), "admitted": True})
            except Exception as exc:  # noqa: BLE001
                upload_log.append({"key": f"up{j}", "admitted": False, "error": str(exc)[:120]})

    up = threading.Thread(target=uploader, daemon=True)
    up.start()
    reqs, full = served_phase(20000.0, 41)
    stop_uploads.set()
    up.join(timeout=30)
    low_rate = float(os.environ.get("QHMAT_GB300_SERVE_LOW_RATE", "3000"))
    _, low = served_phase(low_rate, 42)
    # the load curve between the sustained and the offered rate
    by_rate = {}
    for j, mid in enumerate((6000.0, 10000.0, 14000.0)):
        _, by_rate[str(int(mid))] = served_phase(mid, 43 + j)
    engine.stop(drain=True, timeout=120.0)
    base_full = plain_phase(20000.0, 41, float(os.environ.get("QHMAT_GB300_SERVE_PLAIN_S", "20")))
    base_low = plain_phase(low_rate, 42, 60.0)
    served = full
    rhs_per_s = full["rhs_per_s"]

    # same y alone as in the mix: recompute some served requests alone
    worst = 0.0
    for r in reqs[:: max(1, len(reqs) // 24)][:24]:
        if not r.done or r.error:
            continue
        res = pool.get(r.key)
        x = res.x_host[:, r.col:r.col + r.k].numpy()
        y_mix = res.y_host[:, r.col:r.col + r.k].numpy().copy()
        y_plain = res.plain.matmul(np.ascontiguousarray(x))
        g = precision_gate(y_mix, y_plain, x, res.plain.reconstruction_bound)
        worst = max(worst, g["worst_ratio"])
    rate = 20000.0
    out = {
        "metric": "serving RHS/s (continuous batching) and p50/p99 request latency", "value": round(rhs_per_s, 1),
        "unit": "RHS/s", "n_gpus": 1, "steps": len(reqs), "warmup": 0, "ms_per_step": served.get("mean_ms"),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64 plain / f16-limb precision form per matrix calibration",
        "data": "synthetic (seeded points and right-hand sides; matrices constructed on the host)",
        "config": {"workload": f"cfg5: {WORKLOADS['cfg5']['desc']}", "offered_rate": rate, "duration_s": T,
                   "construction_s": round(build_s, 1),
                   "matrices": [dict(sp, effective_tol=b[1], attempts=b[2]) for sp, b in zip(specs, built[:16])]},
        "latency_at_20k": full, "latency_sustained": low, "latency_by_offered_rate": by_rate,
        "plain_per_request_at_20k": base_full, "plain_per_request_sustained": base_low,
        "forms": forms, "hbm_resident_bytes": pool.used_bytes, "uploads": upload_log,
        "mix_gate_worst_ratio": worst,
        "e2e": {"value": round(rhs_per_s, 1), "unit": "RHS/s", "h2d_bytes_per_step": None,
                "d2h_bytes_per_step": None,
                "transfer": "request columns read from and results written to pinned host memory by the "
                            "gather/scatter kernels"},
    }
    print(json.dumps(out), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="cfg2", choices=sorted(WORKLOADS))
    ap.add_argument("--e2e-steps", type=int, default=200)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        raise SystemExit("--warmup must be >= 3")
    if args.impl == "reference":
        return run_reference_arm(args)
    if args.workload in PRECISION_WORKLOADS:
        return run_precision(args)
    if args.workload in SERVING_WORKLOADS:
        return run_serving(args)
    if args.workload in BATCHING_WORKLOADS:
        return run_batching(args)

    world, rank, local = dist_setup()
    import numpy as np

    # Build the matrix (CPU, spawn pool) before the first CUDA call.
    workers = max(1, (os.cpu_count() or 1) // max(1, world))
    data, x, build_s, pts = make_inputs(args.workload, workers, with_points=True)

    import torch

    import qhmat_gb300
    from qhmat_gb300 import _lib

    torch.cuda.set_device(local)
    pg = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
        pg = dist
    lib = _lib.load_library()
    h = qhmat_gb300.HMatrix.from_bytes(data, device=local)
    wl = WORKLOADS[args.workload]
    rhs = wl["rhs"]
    model = h.model_bytes(rhs)
    st = h.stats

    dev = torch.device("cuda", local)
    xd = torch.from_numpy(np.ascontiguousarray(x)).to(dev)
    yd = torch.empty_like(xd)
    need = h.workspace_bytes(rhs)
    ws = torch.empty(need, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    K, W = args.steps, args.warmup
    # phase breakdown: a separate pass with events between the phases (events
    # in the stream stop one kernel from starting under its predecessor's tail,
    # so the timed pass below runs without them)
    KP = min(K, 200)
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(KP)]

    import ctypes as C

    def step_profiled(i):
        arr = (C.c_void_p * 4)(*[e.cuda_event for e in evs[i]])
        rc = lib.qh_matmul_device_profiled(h._h, xd.data_ptr(), yd.data_ptr(), rhs, ws.data_ptr(), need,
                                           stream.cuda_stream, None, arr)
        if rc:
            _lib.raise_for(rc)

    def step():
        rc = lib.qh_matmul_device(h._h, xd.data_ptr(), yd.data_ptr(), rhs, ws.data_ptr(), need,
                                  stream.cuda_stream, None)
        if rc:
            _lib.raise_for(rc)

    def load_for(seconds):
        """Untimed applies for about `seconds` (keeps the GPU busy while the
        clock sampler runs around the timed region)."""
        t0 = time.perf_counter()
        while time.perf_counter() - t0 < seconds:
            for _ in range(50):
                step()
            torch.cuda.synchronize()

    # Events must exist on the device before their handles are recorded.
    for row in evs:
        for e in row:
            e.record(stream)
    torch.cuda.synchronize()
    for i in range(KP):
        step_profiled(i)
    torch.cuda.synchronize()
    for _ in range(W):
        step()
    torch.cuda.synchronize()
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        clk.wait_first()
        load_for(0.6)
        if pg:
            pg.barrier()
        torch.cuda.synchronize()
        t_start.record(stream)
        wall0 = time.perf_counter()
        for _ in range(K):
            step()
        t_end.record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall0
        if pg:
            pg.barrier()
        load_for(0.4)
    total_ms = max_over_ranks(t_start.elapsed_time(t_end), pg, dev)
    ms_step = total_ms / K
    # per-kernel durations (separate pass, events between the phases)
    kern = {"prep_x": [], "column": [], "row": []}
    for i in range(KP):
        e = evs[i]
        kern["prep_x"].append(e[0].elapsed_time(e[1]))
        kern["column"].append(e[1].elapsed_time(e[2]))
        kern["row"].append(e[2].elapsed_time(e[3]))
    kmean = {k: statistics.mean(v) for k, v in kern.items()}
    # algorithmic bytes per launch of each phase (the packed-byte model split
    # by side): prep (x gathered, exponent, limbs), column (column kernel: Q
    # codes, two scales, the dense diagonal blocks), row (row kernel +
    # combine: P codes, y written)
    n = h.order
    comps = st["components"]
    alg = {
        "prep_x": 8 * n * rhs,
        "column": st["right_code_bytes"] + 16 * comps + st["dense_bytes"],
        "row": st["left_code_bytes"] + 8 * n * rhs,
    }
    dom = max(kmean, key=lambda k: kmean[k])
    peak, peak_src = measured_peak()
    achieved = alg[dom] / (kmean[dom] * 1e-3) / 1e9
    traffic_file = ROOT / "profiles" / f"traffic_{args.workload}.json"
    traffic = None
    if traffic_file.exists():
        try:
            traffic = json.loads(traffic_file.read_text()).get(dom)
        except ValueError:
            traffic = None
    value = whole_job_gbs(model, world, ms_step)

    y_gpu = yd.cpu().numpy()
    out = {
        "metric": METRIC, "value": round(value, 2), "unit": "GB/s",
        "n_gpus": world, "steps": K, "warmup": W, "ms_per_step": round(ms_step, 5),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64 (int2..int32 codes x 62-bit fixed-point x/u, exact f16 tensor-core digit x limb products; "
                 "FP64 scales, diagonal)",
        "data": DATA_NOTE,
        "config": _config(args.workload, wl), "construction_s": round(build_s, 1),
        "workload_stats": {"parallelism": f"replicas x{world}", "model_bytes": model, "components": comps,
                           "blocks": st["block_count"]},
        "pct_hbm_peak": round(100 * value / world / peak, 1),
        "rhs_per_s": round(rhs * world / (ms_step * 1e-3), 1),
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak,
                     "unit": "GB/s", "frac": round(achieved / peak, 4), "traffic": traffic,
                     "peak_source": peak_src, "algorithmic_bytes": alg[dom],
                     "kernel_ms": {k: round(v, 5) for k, v in kmean.items()},
                     "whole_apply_frac": round(value / world / peak, 4)},
        "gpu_launches": int(st["launches_per_apply"]) * K,
        "clocks": clk.summary(),
        "wall_ms_per_step": round(1e3 * wall / K, 5),
    }
    if rank == 0:
        # e2e: host buffers through qh_matmul_host (x in, apply, y out, timed)
        xh = np.ascontiguousarray(x)
        for _ in range(3):
            h.matmul(xh)
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            y_host = h.matmul(xh)
        e2e_s = (time.perf_counter() - t0) / args.e2e_steps
        out["e2e"] = {"value": round(model / e2e_s / 1e9, 2), "unit": "GB/s",
                      "h2d_bytes_per_step": int(xh.nbytes), "d2h_bytes_per_step": int(y_host.nbytes),
                      "ms_per_step": round(1e3 * e2e_s, 4),
                      "transfer": ("x read and y written by the kernels in host memory over the coherent "
                                   "host link" if st["host_direct"] else
                                   "pinned staging: H2D copy of x, D2H copy of y")}
        out["accuracy"] = dense_oracle_error(pts, wl["kernel"], x, y_gpu, dev)
        out["accuracy"]["reconstruction_bound"] = h.reconstruction_bound
        if not args.no_cpu_baseline:
            base, y_cpu = cpu_baseline(data, x, model)
            out["cpu_baseline"] = base
            err = float(np.linalg.norm(y_gpu - y_cpu) / np.linalg.norm(y_cpu))
            out["parity"] = {"rel_err_vs_oracle": err, "tolerance": 1e-13,
                             "host_path_equals_device_path": bool(np.array_equal(y_host, y_gpu))}
        print(json.dumps(out), flush=True)
    if pg:
        pg.barrier()
        pg.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
