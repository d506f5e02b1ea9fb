"""Learned tuner on the CPU: the oracle's gradients against finite
differences, and the committed network (faz_gb300/tuner_mlp.npz) against the
committed training set of QoZ-tuner labels, evaluated with the oracle's
forward pass (no GPU)."""
import os

import numpy as np
import pytest

import faz_gb300.learned as L
import oracle.mlp_oracle as M

HERE = os.path.dirname(os.path.abspath(__file__))
DATA = os.path.join(os.path.dirname(HERE), "faz_gb300", "tuner_c4_dataset.npz")


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = rng.standard_normal(M.N_PARAMS) * 0.1
    X = rng.standard_normal((6, 64))
    lab = np.full((6, 8), -1)
    for h, (lo, n) in enumerate(M.HEADS):
        lab[:, h] = rng.integers(-1, n, size=6)
    _, g = M.loss_and_grad(p, X, lab)
    for idx in [3, 16384 + 5, 16640 + 1000, 82176 + 3, 82432 + 77, 89344 + 26, 500, 17000]:
        e = 1e-6
        pp = p.copy()
        pp[idx] += e
        l1 = M.loss_and_grad(pp, X, lab)[0].mean()
        pp[idx] -= 2 * e
        l2 = M.loss_and_grad(pp, X, lab)[0].mean()
        assert abs((l1 - l2) / (2 * e) - g[idx]) <= 1e-6 + 1e-5 * abs(g[idx])


def test_parameter_layout_matches_header():
    assert L.N_PARAMS == M.N_PARAMS == 89371
    assert L.HEADS == M.HEADS
    assert sum(n for _, n in L.HEADS) == L.N_LOGITS


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 65504.0], np.float32)
    assert list(M.bf16(x)) == [1.0, 1.0, 1.0 + 2 ** -6, -2.5, 65536.0]


@pytest.mark.skipif(not os.path.exists(L.DEFAULT_MODEL) or not os.path.exists(DATA), reason="no committed model")
def test_committed_network_beats_the_majority_rule_on_held_out_fields():
    """What the trained network gains over the method without it: per head,
    its accuracy on the QoZ tuner's decisions for the validation fields (the
    1/8 of the dataset training never saw) against always answering the most
    frequent decision; the accuracies recorded with the model are these."""
    d = np.load(DATA)
    X, Y = d["X"], d["Y"]
    _, va = L.split(len(X))
    m = L.TunerModel.load()
    z = M.forward(m.params, (X[va] - m.mean) / m.std)[2]
    acc = L.head_accuracy(z, Y[va])
    majority = L.majority_rates(Y[va])
    for h in range(L.N_HEADS):
        assert acc[h] >= majority[h] - 1e-9, (h, acc[h], majority[h])
    # the per-level interpolator / direction heads carry the tuner's decisions
    for h in range(4):
        assert acc[h] >= majority[h] + 0.15, (h, acc[h], majority[h])
    assert np.mean(acc[:4]) > 0.85, acc
    rec = np.load(L.DEFAULT_MODEL)
    if "val_accuracy" in rec.files:
        assert np.allclose(rec["val_accuracy"], acc, atol=0.01), (rec["val_accuracy"], acc)


@pytest.mark.skipif(not os.path.exists(L.DEFAULT_MODEL), reason="no committed model")
def test_committed_network_bf16_inference_agrees_with_fp64():
    d = np.load(DATA)
    m = L.TunerModel.load()
    X = d["X"][:256]
    z64 = M.forward(m.params, (X - m.mean) / m.std)[2]
    z16 = M.infer_bf16(m.params, m.mean, m.std, X)
    agree = (L.head_predictions(z64) == L.head_predictions(z16)).mean()
    assert agree > 0.98, agree
