"""Host logic of the form calibration, on CPU with stand-ins for the two
forms: the precision form is tried with two-chunk accumulation segments and
then one-chunk segments before the plain form is chosen, in a single handle
(choose_form) and across a batch (batch_forms)."""

import numpy as np

from qhmat_gb300.batching import batch_forms
from qhmat_gb300.matrix import choose_form


class _Plain:
    """A stand-in plain form: y = A x for a small dense A."""

    def __init__(self, a, bound):
        self.a = a
        self.order = a.shape[0]
        self.reconstruction_bound = bound

    def matmul(self, x):
        return self.a @ x


class _Precision:
    """A stand-in precision form whose deviation from the plain form is
    ``err[segment_chunks]`` times 0.01 bound ||x||_1 (so the gate ratio is
    err[...] exactly)."""

    def __init__(self, plain, err):
        self.plain = plain
        self.err = err
        self.segment_chunks = 2

    def matmul(self, x):
        y = self.plain.matmul(x)
        dev = 0.01 * self.plain.reconstruction_bound * np.sum(np.abs(x), axis=0) * self.err[self.segment_chunks]
        y = y.copy()
        y[0] += dev
        return y


def _forms(err):
    rng = np.random.default_rng(0)
    plain = _Plain(rng.standard_normal((40, 40)), 1e-6)
    pf = _Precision(plain, err)
    return choose_form(plain, pf, probes=4), pf


def test_default_segments_when_they_pass():
    g, pf = _forms({2: 0.3, 1: 0.1})
    assert g["form"] == "precision" and g["segment_chunks"] == 2 and pf.segment_chunks == 2
    assert abs(g["worst_ratio"] - 0.3) < 1e-9


def test_falls_back_to_one_chunk_segments():
    g, pf = _forms({2: 0.9, 1: 0.4})
    assert g["form"] == "precision" and g["segment_chunks"] == 1 and pf.segment_chunks == 1
    assert abs(g["worst_ratio"] - 0.4) < 1e-9


def test_plain_when_neither_passes_and_default_restored():
    g, pf = _forms({2: 3.0, 1: 1.2})
    assert g["form"] == "plain" and pf.segment_chunks == 2


def test_batch_forms():
    # no matrix needs one-chunk segments: judged at two
    assert batch_forms([0.1, 0.9, 0.2], [0.05, 0.6, 0.1], [4, 4, 4]) == (2, ["precision", "plain", "precision"])
    # the second passes only with one-chunk segments: the whole batch uses them
    assert batch_forms([0.1, 0.9, 3.0], [0.05, 0.4, 1.5], [4, 4, 4]) == (1, ["precision", "precision", "plain"])
    # single-column matrices stay plain and do not force one-chunk segments
    assert batch_forms([0.1, 0.9], [0.05, 0.4], [4, 1]) == (2, ["precision", "plain"])
