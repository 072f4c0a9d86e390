"""Construction of quantized H-matrices (host side, CPU, parallel over blocks).

A restatement of the reference's construction so that matrices of the sizes
the GPU apply is measured on can be built where the reference is not
installed, written in the reference's own file format (QHMAT001):

* ``spatial_partition``  -- src/qhmat/core.cpp:117-203 (median split on the
  widest axis, bounding-box admissibility ``dist >= eta * diam``);
* ``coefficient`` / ``allocate`` -- src/qhmat/core.cpp:56-115 (reserve-greedy,
  tail-first bit allocation; sums in the platform's ``long double``);
* ``from_kernel`` -- HMatrix.from_partition (python/qhmat/matrix.py:153-251)
  applied to a kernel matrix whose entries are evaluated block by block from
  the points (the same values ``from_dense`` would read from the full array);
* ``pack`` -- HMatrix::pack (src/qhmat/core.cpp:235-267) with the balanced
  factors of HMatrix::add_low_rank (src/qhmat/core.cpp:284-330);
* ``to_qhmat_bytes`` -- the QHMAT001 layout (src/qhmat/io.cpp:139-163).

Blocks are independent, so they are built in a pool of worker processes
(``spawn`` start method, one BLAS thread each); results are assembled in block
order, so the output does not depend on the worker count.  On the same
machine and NumPy build the bytes equal those of the reference's
``HMatrix.from_dense(...).save()`` (checked by tests/test_construct.py).
"""

from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np


class InfeasibleError(ValueError):
    """A non-diagonal block cannot meet its truncation or bit-allocation budget."""


# ----------------------------------------------------------------- kernels

def kernel_inverse(r):
    """A = 1 / (r + 0.4)."""
    return 1.0 / (r + 0.4)


def kernel_log(r):
    """A = -log(r + 1e-3)."""
    return -np.log(r + 1e-3)


def kernel_yukawa(r):
    """A = exp(-r) / (r + 0.05)."""
    return np.exp(-r) / (r + 0.05)


KERNELS = {"inverse": kernel_inverse, "log": kernel_log, "yukawa": kernel_yukawa}


def distances(p: np.ndarray, q: np.ndarray) -> np.ndarray:
    """Euclidean distances between rows of p and rows of q (|pi - qj| in 1-D)."""
    if p.shape[1] == 1:
        return np.abs(p[:, 0][:, None] - q[:, 0][None, :])
    return np.sqrt(((p[:, None, :] - q[None, :, :]) ** 2).sum(-1))


def kernel_matrix(points: np.ndarray, kernel: str) -> np.ndarray:
    """The dense kernel matrix (small cases; from_kernel never forms it)."""
    return KERNELS[kernel](distances(points, points))


# --------------------------------------------------------------- partition

@dataclass
class _Cluster:
    first: int
    last: int = 0
    lower: np.ndarray = field(default=None)
    upper: np.ndarray = field(default=None)
    left: int = -1
    right: int = -1


def spatial_partition(points, leaf_size: int, admissibility: float = 1.0,
                      support_lower=None, support_upper=None):
    """Return (permutation, blocks) with blocks as (row0, row1, col0, col1, admissible)."""
    pts = np.ascontiguousarray(points, dtype=np.float64)
    if pts.ndim != 2 or pts.shape[0] == 0 or not 0 < pts.shape[1] <= 16:
        raise ValueError("invalid point-cloud dimensions")
    lo = pts if support_lower is None else np.asarray(support_lower, np.float64)
    hi = pts if support_upper is None else np.asarray(support_upper, np.float64)
    if lo.shape != pts.shape or hi.shape != pts.shape:
        raise ValueError("point/support shapes differ")
    if leaf_size <= 0 or not math.isfinite(admissibility) or admissibility <= 0:
        raise ValueError("leaf size and admissibility must be positive")
    if not (np.isfinite(pts).all() and np.isfinite(lo).all() and np.isfinite(hi).all()
            and (lo <= pts).all() and (pts <= hi).all()):
        raise ValueError("invalid point or support box")
    dim = pts.shape[1]
    perm: list[int] = []
    tree: list[_Cluster] = []

    def build(indices: np.ndarray) -> int:
        c = _Cluster(first=len(perm))
        c.lower = lo[indices].min(axis=0)
        c.upper = hi[indices].max(axis=0)
        cid = len(tree)
        tree.append(c)
        if indices.size <= leaf_size:
            perm.extend(int(i) for i in indices)
        else:
            span = pts[indices].max(axis=0) - pts[indices].min(axis=0)
            axis = 0
            for d in range(1, dim):
                if span[d] > span[axis]:
                    axis = d
            order = np.argsort(pts[indices, axis], kind="stable")
            srt = indices[order]
            mid = srt.size // 2
            left = build(srt[:mid])
            right = build(srt[mid:])
            tree[cid].left, tree[cid].right = left, right
        tree[cid].last = len(perm)
        return cid

    root = build(np.arange(pts.shape[0]))
    norms = [math.sqrt(sum((float(c.upper[d]) - float(c.lower[d])) ** 2 for d in range(dim)))
             for c in tree]
    blocks: list[tuple[int, int, int, int, bool]] = []

    def visit(ai: int, bi: int) -> None:
        a, b = tree[ai], tree[bi]
        d2 = 0.0
        for d in range(dim):
            gap = max(0.0, float(a.lower[d]) - float(b.upper[d]), float(b.lower[d]) - float(a.upper[d]))
            d2 += gap * gap
        dist = math.sqrt(d2)
        diam = max(norms[ai], norms[bi])
        adm = dist > 0.0 and dist >= admissibility * diam
        if adm or (a.left < 0 and b.left < 0):
            blocks.append((a.first, a.last, b.first, b.last, adm))
            return
        aa = [ai] if a.left < 0 else [a.left, a.right]
        bb = [bi] if b.left < 0 else [b.left, b.right]
        for x in aa:
            for y in bb:
                visit(x, y)

    visit(root, root)
    return np.asarray(perm, dtype=np.int64), blocks


# -------------------------------------------------------------- allocation

def coefficient(bits: int) -> float:
    """c(b) = 1/q + 1/(4 q^2), q = 2^(b-1) - 1."""
    if not 2 <= bits <= 32:
        raise ValueError("bit width must be in [2, 32]")
    q = float((1 << (bits - 1)) - 1)
    return 1.0 / q + 1.0 / (4.0 * q * q)


def allocate(sigma, bit_widths, budget: float, rows: int, cols: int):
    """Per-component widths meeting sum_j sigma_j c(b_j) <= budget.

    Returns (bits, bound, payload_bits, feasible)."""
    if rows <= 0 or cols <= 0:
        raise ValueError("matrix dimensions must be positive")
    if not math.isfinite(budget) or budget < 0:
        raise ValueError("budget must be finite and nonnegative")
    s = [float(v) for v in np.asarray(sigma, dtype=np.float64).ravel()]
    menu = sorted(int(b) for b in bit_widths)
    if not menu or len(set(menu)) != len(menu):
        raise ValueError("precision menu must be non-empty and free of duplicates")
    for b in menu:
        coefficient(b)
    LD = np.longdouble
    rank = len(s)
    prefix = [LD(0)] * (rank + 1)
    for j in range(rank):
        prefix[j + 1] = prefix[j] + LD(s[j])
    high = LD(coefficient(menu[-1]))
    bits = [menu[-1]] * rank
    if high * prefix[rank] <= LD(budget):
        remaining = rank
        available = LD(budget)
        for level in range(len(menu) - 1):
            c = LD(coefficient(menu[level]))
            channel = LD(0)
            while remaining:
                nxt = channel + c * LD(s[remaining - 1]) + high * prefix[remaining - 1]
                if nxt > available:
                    break
                bits[remaining - 1] = menu[level]
                channel += c * LD(s[remaining - 1])
                remaining -= 1
            available -= channel
    bound = LD(0)
    for j in range(rank):
        bound += LD(s[j]) * LD(coefficient(bits[j]))
    payload = (rows + cols) * sum(bits)
    return bits, float(bound), payload, bool(bound <= LD(budget))


# -------------------------------------------------------------------- pack

def pack(matrix: np.ndarray, widths) -> tuple[np.ndarray, np.ndarray]:
    """Quantize and bit-pack the columns of a (rows, rank) FP64 factor.

    Returns (words uint32, scales float64); component runs are consecutive and
    each starts at a fresh word."""
    rows, rank = matrix.shape
    scales = np.zeros(rank, np.float64)
    runs = []
    for j in range(rank):
        b = int(widths[j])
        q = (1 << (b - 1)) - 1
        col = matrix[:, j]
        maximum = float(np.max(np.abs(col))) if rows else 0.0
        scale = 0.0 if maximum == 0 else maximum / float(q)
        scales[j] = scale
        nwords = (rows * b + 31) // 32
        if scale == 0:
            runs.append(np.zeros(nwords, np.uint32))
            continue
        codes = np.clip(np.rint(col / scale).astype(np.int64), -q, q)
        raw = (codes & ((1 << b) - 1)).astype(np.uint64)
        pos = np.arange(rows, dtype=np.int64) * b
        word = pos >> 5
        val = raw << (pos & 31).astype(np.uint64)
        # fields never overlap, so summing the pieces equals OR-ing them
        lo = np.bincount(word, weights=(val & np.uint64(0xFFFFFFFF)).astype(np.float64),
                         minlength=nwords + 1)
        hi = np.bincount(word + 1, weights=(val >> np.uint64(32)).astype(np.float64),
                         minlength=nwords + 1)
        runs.append((lo + hi)[:nwords].astype(np.uint64).astype(np.uint32))
    words = np.concatenate(runs) if runs else np.zeros(0, np.uint32)
    return words, scales


# ----------------------------------------------------------- construction

@dataclass
class Block:
    row0: int
    row1: int
    col0: int
    col1: int
    admissible: bool
    dense: np.ndarray | None = None
    widths: list = field(default_factory=list)
    menu_size: int = 0
    truncation_error: float = 0.0
    quantization_bound: float = 0.0
    left_scales: np.ndarray | None = None
    right_scales: np.ndarray | None = None
    left_words: np.ndarray | None = None
    right_words: np.ndarray | None = None

    @property
    def rank(self) -> int:
        return len(self.widths)


@dataclass
class Image:
    """A constructed matrix: permutation plus blocks in insertion order."""
    order: int
    permutation: np.ndarray
    blocks: list

    @property
    def reconstruction_bound(self) -> float:
        return max((b.truncation_error + b.quantization_bound for b in self.blocks), default=0.0)


def _randomized_svd(blk, rect, l=96, power=2):
    """Rank-l SVD of a block by a seeded randomized range finder (``power``
    subspace iterations), and the tails tail[r] = ||blk - blk_r||_F for
    r <= l, computed from the explicit residual of the rank-l factors plus
    the dropped singular values (no cancellation)."""
    m, n = blk.shape
    rng = np.random.default_rng((int(rect[0]) * 1000003 + int(rect[2])) & 0x7FFFFFFF)
    y = blk @ rng.standard_normal((n, l))
    for _ in range(power):
        y, _ = np.linalg.qr(y)
        y = blk @ (blk.T @ y)
    q, _ = np.linalg.qr(y)
    ub, sigma, vt = np.linalg.svd(q.T @ blk, full_matrices=False)
    u = q @ ub
    resid = blk - (u * sigma) @ vt
    r2 = float(np.sum(resid * resid))
    tail = np.sqrt(r2 + np.r_[np.cumsum((sigma[::-1] ** 2))[::-1], 0.0])
    return u, sigma, vt, tail


def _build_block(pts, perm, rect, kernel, tolerance, widths, rank_tol, max_rank, trunc, reserve, svd="exact"):
    row0, row1, col0, col1, adm = rect
    kfn = KERNELS[kernel]
    blk = np.ascontiguousarray(kfn(distances(pts[perm[row0:row1]], pts[perm[col0:col1]])))
    out = Block(row0, row1, col0, col1, adm)
    if row0 == col0 and row1 == col1:
        out.dense = blk
        return out
    if not (row1 <= col0 or col1 <= row0):
        raise ValueError("non-diagonal block intersects the diagonal")
    out.menu_size = len(widths)
    budget = tolerance * float(np.max(np.abs(blk)))
    m, n = blk.shape
    if budget == 0.0:
        out.left_scales, out.right_scales = np.zeros(0), np.zeros(0)
        out.left_words, out.right_words = np.zeros(0, np.uint32), np.zeros(0, np.uint32)
        return out
    rank = None
    if svd == "randomized" and min(m, n) > 128:
        # fast path for large blocks: a rank-96 randomized SVD; the rank rule
        # on its (never smaller) tails, the residual measured exactly below
        u, sigma, vt, tail = _randomized_svd(blk, rect)
        full = float(np.sqrt(np.sum(blk * blk)))
        target = min(rank_tol * full, trunc * budget)
        cap = sigma.size if max_rank is None else min(max_rank, sigma.size)
        rank = next((r for r in range(1, cap + 1) if tail[r] <= target), None)
    if rank is None:
        u, sigma, vt = np.linalg.svd(blk, full_matrices=False)
        tail = np.sqrt(np.r_[np.cumsum((sigma[::-1] ** 2))[::-1], 0.0])
        target = min(rank_tol * tail[0], trunc * budget)
        cap = sigma.size if max_rank is None else min(max_rank, sigma.size)
        rank = next((r for r in range(1, cap + 1) if tail[r] <= target), None)
    if rank is None:
        raise InfeasibleError(f"block ({row0}:{row1}, {col0}:{col1}) cannot satisfy the truncation allowance")
    rank = min(rank, int(np.count_nonzero(sigma > 0)))
    sigma = sigma[:rank]
    u = u[:, :rank]
    v = vt[:rank, :].T
    residual = float(np.max(np.abs(blk - (u * sigma) @ v.T)))
    q_budget = budget * (1 - reserve) - residual
    if residual > trunc * budget or q_budget < 0:
        raise InfeasibleError("measured truncation error exceeds the block allowance")
    bits, _, _, feasible = allocate(sigma, widths, q_budget, m, n)
    if not feasible:
        raise InfeasibleError(f"block ({row0}:{row1}, {col0}:{col1}) is infeasible even at the highest bit width")
    # balanced factors and quantization bound, in component order
    qb = 0.0
    for j in range(rank):
        qb += float(sigma[j]) * coefficient(bits[j])
    root = np.sqrt(sigma)
    out.widths = [int(b) for b in bits]
    out.truncation_error = residual
    out.quantization_bound = qb
    out.left_words, out.left_scales = pack(u * root, bits)
    out.right_words, out.right_scales = pack(v * root, bits)
    return out


_WORKER = {}


def _worker_init(pts, perm, kernel, tolerance, widths, rank_tol, max_rank, trunc, reserve, svd="exact"):
    _WORKER.update(pts=pts, perm=perm, args=(kernel, tolerance, widths, rank_tol, max_rank, trunc, reserve, svd))


def _worker_run(rects):
    w = _WORKER
    try:
        return [_build_block(w["pts"], w["perm"], r, *w["args"]) for r in rects]
    except InfeasibleError as exc:
        return exc


def from_kernel_escalating(points, kernel: str, *, tolerance: float, leaf_size: int = 32,
                           step: float = 10 ** 0.25, max_attempts: int = 40, probe_blocks: int = 256, **kw):
    """``from_kernel`` at ``tolerance``, multiplied by ``step`` after every
    InfeasibleError until the construction succeeds (the deterministic
    escalation rule of the batched and served workloads).  Each attempt first
    builds the first ``probe_blocks`` blocks of the partition in this process
    (the finest near-diagonal blocks, where an infeasible tolerance fails
    first), so a failing attempt costs no worker pool.  Returns (image,
    effective tolerance, attempts)."""
    pts = np.ascontiguousarray(points, dtype=np.float64)
    perm, rects = spatial_partition(pts, leaf_size, kw.get("admissibility", 1.0))
    widths = tuple(int(b) for b in kw.get("bit_widths", (4, 8, 12, 16, 24, 32)))
    tol = tolerance
    for attempt in range(1, max_attempts + 1):
        args = (kernel, tol, widths, kw.get("rank_tolerance", 0.1), kw.get("max_rank"),
                kw.get("truncation_fraction", 0.25), kw.get("arithmetic_reserve", 0.02), kw.get("svd", "exact"))
        try:
            for r in rects[:probe_blocks]:
                _build_block(pts, perm, r, *args)
            return from_kernel(pts, kernel, tolerance=tol, leaf_size=leaf_size, **kw), tol, attempt
        except InfeasibleError:
            tol *= step
    raise InfeasibleError(f"no feasible tolerance within {max_attempts} escalations of {tolerance}")


def from_kernel(points, kernel: str, *, tolerance: float, leaf_size: int = 32,
                admissibility: float = 1.0, bit_widths=(4, 8, 12, 16, 24, 32),
                rank_tolerance: float = 0.1, max_rank: int | None = None,
                truncation_fraction: float = 0.25, arithmetic_reserve: float = 0.02,
                workers: int | None = None, svd: str = "exact") -> Image:
    """Build the quantized H-matrix of ``KERNELS[kernel](|p_i - p_j|)``.

    With ``svd="exact"`` (default): the same parameters and results as the
    reference's ``HMatrix.from_dense`` on the dense kernel matrix; raises
    :class:`InfeasibleError` likewise.  ``svd="randomized"`` is the fast path
    for large workloads: blocks wider than 128 take a seeded rank-96
    randomized SVD (the exact one when rank 96 does not meet the block's
    target), so factors and codes differ from the reference's in their low
    bits while every block still passes the same measured-residual and
    bit-allocation checks."""
    pts = np.ascontiguousarray(points, dtype=np.float64)
    if kernel not in KERNELS:
        raise ValueError(f"unknown kernel {kernel!r}")
    if not math.isfinite(tolerance) or tolerance <= 0:
        raise ValueError("tolerance must be finite and positive")
    widths = tuple(int(b) for b in bit_widths)
    if not widths or any(not 2 <= b <= 32 for b in widths) or len(set(widths)) != len(widths):
        raise ValueError("bit_widths must contain distinct integers in [2, 32]")
    perm, rects = spatial_partition(pts, leaf_size, admissibility)
    if svd not in ("exact", "randomized"):
        raise ValueError("svd must be 'exact' or 'randomized'")
    args = (kernel, tolerance, widths, rank_tolerance, max_rank, truncation_fraction, arithmetic_reserve, svd)
    workers = workers if workers is not None else min(os.cpu_count() or 1, 16)
    if workers <= 1 or len(rects) < 64:
        blocks = [_build_block(pts, perm, r, *args) for r in rects]
        return Image(pts.shape[0], perm, blocks)
    # Balance by cost (~ m*n*min(m,n)), in contiguous chunks to keep order.
    import multiprocessing as mp

    cost = np.array([(r[1] - r[0]) * (r[3] - r[2]) * min(r[1] - r[0], r[3] - r[2]) for r in rects], float)
    nchunks = workers * 8
    bounds = np.searchsorted(np.cumsum(cost), np.linspace(0, cost.sum(), nchunks + 1)[1:-1])
    chunks = [c.tolist() for c in np.split(np.arange(len(rects)), bounds) if c.size]
    env = {k: os.environ.get(k) for k in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS")}
    for k in env:
        os.environ[k] = "1"
    try:
        ctx = mp.get_context("spawn")
        results = []
        with ctx.Pool(workers, initializer=_worker_init, initargs=(pts, perm, *args)) as pool:
            # in block order; the first infeasible chunk ends the construction
            for res in pool.imap(_worker_run, [[rects[i] for i in c] for c in chunks], chunksize=1):
                if isinstance(res, Exception):
                    pool.terminate()
                    raise res
                results.append(res)
    finally:
        for k, v in env.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    blocks = []
    for res in results:
        blocks.extend(res)
    return Image(pts.shape[0], perm, blocks)


# ----------------------------------------------------------------- writer

def _u64(v) -> bytes:
    return int(v).to_bytes(8, "little")


def to_qhmat_bytes(img: Image, checksum=None) -> bytes:
    """Serialise in QHMAT001 (little-endian, FNV-1a-64 trailer).

    ``checksum(body) -> int`` computes the trailer; by default the library's
    ``qh_fnv1a64``."""
    parts = [b"QHMAT001", _u64(1), _u64(img.order), _u64(len(img.blocks)),
             np.asarray(img.permutation, dtype="<u8").tobytes()]
    for b in img.blocks:
        parts.append(np.array([b.row0, b.row1, b.col0, b.col1], dtype="<u8").tobytes())
        parts.append(bytes([1 if b.admissible else 0, 0 if b.dense is None else 1]))
        if b.dense is not None:
            parts.append(np.ascontiguousarray(b.dense, dtype="<f8").tobytes())
            continue
        parts.append(_u64(b.rank) + _u64(b.menu_size))
        parts.append(np.array([b.truncation_error, b.quantization_bound], dtype="<f8").tobytes())
        parts.append(bytes(b.widths))
        parts.append(np.asarray(b.left_scales, dtype="<f8").tobytes())
        parts.append(np.asarray(b.right_scales, dtype="<f8").tobytes())
        parts.append(np.asarray(b.left_words, dtype="<u4").tobytes())
        parts.append(np.asarray(b.right_words, dtype="<u4").tobytes())
    body = b"".join(parts)
    if checksum is None:
        from ._lib import load_library

        def checksum(b):
            return load_library().qh_fnv1a64(b, len(b))

    return body + int(checksum(body)).to_bytes(8, "little")
