"""Host logic of the serving form on CPU: HBM admission accounting (LRU
eviction of idle matrices, pinned matrices kept, refusal when nothing fits)
and the seeded workload generators with the tolerance-escalation rule."""

import pytest

import bench
from qhmat_gb300.serving import AdmissionController, AdmissionError


def test_admission_evicts_least_recently_used_idle_matrices():
    a = AdmissionController(100)
    for k, sz in (("a", 30), ("b", 30), ("c", 30)):
        assert a.reserve(k, sz) == []
        a.commit(k, sz)
    a.touch("a")  # b is now the least recently used
    victims = a.reserve("d", 40)  # 10 free; evicting b frees 40
    assert victims == ["b"]
    for v in victims:
        a.release(v)
    a.commit("d", 40)
    assert a.used <= a.budget


def test_admission_keeps_pinned_and_refuses():
    a = AdmissionController(100)
    a.commit("a", 60)
    a.commit("b", 30)
    a.pin("a")
    a.pin("b")
    with pytest.raises(AdmissionError):
        a.reserve("c", 50)  # both resident matrices are in use
    a.unpin("b")
    assert a.reserve("c", 20) == ["b"]
    with pytest.raises(AdmissionError, match="whole budget"):
        a.reserve("z", 101)
    with pytest.raises(ValueError, match="already resident"):
        a.reserve("a", 1)


def test_matrix_specs_are_seeded_and_in_range():
    s1 = bench.matrix_specs(64, 3)
    assert s1 == bench.matrix_specs(64, 3)
    for sp in s1:
        assert 512 <= sp["n"] <= 8192 and sp["dim"] in (1, 2) and sp["leaf"] in (16, 32, 64)
        assert 1e-8 <= sp["tol"] <= 1e-4 and 1 <= sp["rhs"] <= 32 and sp["kernel"] in ("inverse", "log")
    s5 = bench.matrix_specs(8, 4, n_values=(1024, 4096))
    assert [sp["n"] for sp in s5] == [1024, 4096] * 4


def test_tolerance_escalation_reaches_a_feasible_tolerance():
    """1e-8 is infeasible for these kernels; the rule multiplies by 10^0.25
    until the construction succeeds, and the result is reproducible."""
    from oracle import oracle as O

    spec = dict(n=600, dim=1, kernel="log", tol=1e-8, leaf=32, rhs=3, seed=7)
    data, tol, attempts = bench.build_spec(spec, 1, checksum=O.fnv1a64)
    assert attempts > 1 and tol > 1e-8
    assert abs(tol / 1e-8 - 10 ** (0.25 * (attempts - 1))) < 1e-6 * tol / 1e-8
    assert bench.build_spec(spec, 1, checksum=O.fnv1a64)[0] == data
    m = O.OracleMatrix(data)
    assert m.order == 600


def test_device_bytes_query_needs_no_device():
    """The admission size query parses the image and builds the layouts on
    the host (no device): positive sizes, the precision form's only when
    asked for, and the loader's errors for a corrupt image."""
    from conftest import golden
    from qhmat_gb300 import qhmat_device_bytes

    data, _ = golden("cfg1")
    plain, pf = qhmat_device_bytes(data, sms=152)
    assert plain > 0 and pf > 0
    assert qhmat_device_bytes(data, sms=152, precision=False) == (plain, 0)
    with pytest.raises((ValueError, RuntimeError)):
        qhmat_device_bytes(data[:100], sms=152)
    with pytest.raises(ValueError, match="SM count"):
        qhmat_device_bytes(data, sms=0)
