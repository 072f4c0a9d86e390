"""GPU tests of the serving form: a request's y is the same alone and in a
mix of concurrent requests (bit for bit for the plain form; the precision
form within its acceptance gate), cancelled requests are never applied,
corrupt uploads are rejected without leaking budget, and an upload that does
not fit the HBM budget is refused."""

import time

import numpy as np
import pytest

from conftest import golden, rel_err
from qhmat_gb300 import precision_gate
from qhmat_gb300.serving import AdmissionError, ServingEngine, ServingPool

pytestmark = pytest.mark.gpu


def _wait(reqs, timeout=60.0):
    t0 = time.time()
    while not all(r.done or r.cancelled for r in reqs):
        assert time.time() - t0 < timeout, "requests did not complete"
        time.sleep(0.001)


def test_same_result_alone_and_in_the_mix(cuda_device):
    """120 requests of 1..16 columns over four resident matrices, submitted at
    once (continuous batching on three streams), each in its own columns;
    then every request again alone.  Plain-form matrices: bitwise equal;
    precision-form matrices: within the acceptance gate."""
    import torch

    pool = ServingPool(device=cuda_device, budget_bytes=8 << 30)
    names = ["cfg1", "ragged300", "cuda10", "orth17_b24"]
    rng = np.random.default_rng(4)
    cols = 512
    for name in names:
        data, _ = golden(name)
        r = pool.admit(name, data, columns=cols)
        r.x_host.copy_(torch.from_numpy(rng.standard_normal((r.order, cols))))
    eng = ServingEngine(pool, streams=3, depth=2, max_cols=64, max_order=2048).start()
    nxt = {name: 0 for name in names}
    mix = []
    for i in range(120):
        name = names[i % 4]
        k = int(rng.integers(1, 17))
        mix.append(eng.submit(name, nxt[name], k))
        nxt[name] += k
    _wait(mix)
    assert all(not r.error for r in mix), [r.error for r in mix if r.error][:3]
    assert eng.batches < len(mix)  # requests were batched together
    y_mix = {r.rid: pool.get(r.key).y_host[:, r.col:r.col + r.k].numpy().copy() for r in mix}
    for r in mix:
        rr = eng.submit(r.key, r.col, r.k)
        _wait([rr])
        res = pool.get(r.key)
        y_alone = res.y_host[:, r.col:r.col + r.k].numpy()
        if res.form == "plain":
            assert np.array_equal(y_mix[r.rid], y_alone), r
        else:
            x = res.x_host[:, r.col:r.col + r.k].numpy()
            g = precision_gate(y_mix[r.rid], y_alone, x, res.plain.reconstruction_bound)
            assert g["passes"], (r, g)
    eng.stop()


def test_columns_are_independent_of_batch_composition(cuda_device):
    """The same columns applied in one batch with others and in a batch of
    their own give bitwise equal y (both forms)."""
    import torch

    data, _ = golden("cfg1")
    for precision in (False, True):
        pool = ServingPool(device=cuda_device, budget_bytes=4 << 30, precision=precision)
        r = pool.admit("m", data, columns=64)
        r.x_host.copy_(torch.from_numpy(np.random.default_rng(9).standard_normal((r.order, 64))))
        if precision:
            r.form = "precision"  # force the precision form for multi-column batches
        eng = ServingEngine(pool, streams=1, depth=1, max_cols=64, max_order=2048).start()
        a = eng.submit("m", 0, 40)  # one batch: columns 0..39
        _wait([a])
        y_big = r.y_host[:, 10:14].numpy().copy()
        b = eng.submit("m", 10, 4)  # columns 10..13 alone
        _wait([b])
        eng.stop()
        assert np.array_equal(r.y_host[:, 10:14].numpy(), y_big), precision


def test_cancel_and_corrupt_upload_and_refusal(cuda_device):
    data, g = golden("cfg1")
    pool = ServingPool(device=cuda_device, budget_bytes=1 << 30, precision=False)
    with pytest.raises(RuntimeError, match="checksum mismatch"):
        pool.admit("bad", data[:-9] + bytes([data[-9] ^ 1]) + data[-8:])
    assert pool.used_bytes == 0 and "bad" not in pool.admission
    r = pool.admit("m", data, columns=8)
    r.x_host.copy_(__import__("torch").from_numpy(np.tile(g["x"], (1, 2))))
    eng = ServingEngine(pool, streams=1, depth=1, max_cols=64, max_order=2048)
    req = eng.submit("m", 0, 4)
    assert eng.cancel(req) and req.cancelled
    eng.start()
    req2 = eng.submit("m", 4, 4)
    _wait([req2])
    eng.stop()
    assert not req.done and req2.done
    assert rel_err(r.y_host[:, 4:8].numpy(), g["y"]) <= 1e-13
    small = ServingPool(device=cuda_device, budget_bytes=r.device_bytes - 1, precision=False)
    with pytest.raises(AdmissionError):
        small.admit("m", data)
    assert small.used_bytes == 0


def test_device_bytes_query_matches_uploads(cuda_device):
    """Admission reserves what the host-side size query reports before any
    upload; it must equal what the uploaded handles report."""
    import torch

    from qhmat_gb300 import HMatrix, PrecisionHMatrix, qhmat_device_bytes

    for name in ("cfg1", "ragged300"):
        data, _ = golden(name)
        h = HMatrix.from_bytes(data)
        pm = PrecisionHMatrix.from_bytes(data)
        sms = torch.cuda.get_device_properties(0).multi_processor_count
        assert qhmat_device_bytes(data, sms=sms) == (h.stats["device_bytes"], pm.stats["device_bytes"])
        h.close()
        pm.close()
