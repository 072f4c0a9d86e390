"""GPU tests of the batching form: a block-diagonal batch of independent
matrices applied by one persistent launch chain (and as one CUDA graph).
Plain-form matrices of the batch give exactly their own apply's y (bit for
bit: the per-column power-of-two scaling reproduces each matrix's own fixed
point); precision-form matrices pass the acceptance gate against it; graph
replay equals the eager apply; the autotuner caches its choice."""

import json

import numpy as np
import pytest

from conftest import GOLDEN_CASES, golden
from qhmat_gb300 import HMatrix, precision_gate
from qhmat_gb300.batching import BatchedHMatrices

pytestmark = pytest.mark.gpu


def _inputs(names, seed=3):
    rng = np.random.default_rng(seed)
    images = [golden(n)[0] for n in names]
    rhs = [int(rng.integers(1, 33)) for _ in names]
    return images, rhs, rng


def _own(images, rhs, x_all, offs):
    out = []
    for k, img in enumerate(images):
        h = HMatrix.from_bytes(img)
        x = x_all[offs[k]:offs[k + 1]].reshape(h.order, rhs[k])
        out.append(h.matmul(np.ascontiguousarray(x)).ravel())
        h.close()
    return out


def test_plain_batch_is_bitwise_equal_to_each_matrix(cuda_device):
    import torch

    names = GOLDEN_CASES
    images, rhs, rng = _inputs(names)
    bat = BatchedHMatrices(images, rhs, forms="plain", autotune=False)
    x = rng.standard_normal(bat.total) * np.exp2(rng.integers(-20, 20, bat.total))
    xd = torch.from_numpy(x).cuda()
    yd = torch.zeros_like(xd)
    bat.apply(xd, yd)
    y = yd.cpu().numpy()
    offs = [int(v) for v in bat.x_offsets]
    for k, yk in enumerate(_own(images, rhs, x, offs)):
        assert np.array_equal(y[offs[k]:offs[k + 1]], yk), names[k]
    bat.close()


def test_auto_batch_gate_graph_and_autotune(cuda_device, tmp_path):
    import torch

    names = ["cfg1", "ragged300", "orth17_b32", "orth17_b8", "kernel12", "cuda10"]
    images, rhs, rng = _inputs(names, seed=5)
    cache = tmp_path / "tune.json"
    bat = BatchedHMatrices(images, rhs, forms="auto", autotune=True, cache=cache)
    x = rng.standard_normal(bat.total)
    xd = torch.from_numpy(x).cuda()
    yd = torch.zeros_like(xd)
    bat.apply(xd, yd)
    y_eager = yd.cpu().numpy()
    bat.capture(xd, yd)
    yd.zero_()
    bat.replay()
    torch.cuda.synchronize()
    assert np.array_equal(yd.cpu().numpy(), y_eager)
    offs = [int(v) for v in bat.x_offsets]
    for k, yk in enumerate(_own(images, rhs, x, offs)):
        yb = y_eager[offs[k]:offs[k + 1]]
        if bat.form[k] == "plain":
            assert np.array_equal(yb, yk), names[k]
        else:
            shape = (bat.orders[k], rhs[k])
            g = precision_gate(yb.reshape(shape), yk.reshape(shape), x[offs[k]:offs[k + 1]].reshape(shape),
                               bat.bounds[k])
            assert g["passes"], (names[k], g)
    if "precision" in bat.form:
        table = json.loads(cache.read_text())
        assert bat.tuning["key"] in table and not bat.tuning["cached"]
        again = BatchedHMatrices(images, rhs, forms="auto", autotune=True, cache=cache)
        assert again.tuning["cached"] and again.tuning["grid"] == bat.tuning["grid"]
        again.close()
    bat.close()
