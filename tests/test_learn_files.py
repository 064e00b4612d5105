"""Weights files of the learned form (CPU only): the packaged network and its
training envelope load, and a file without the envelope figure sets no
limit."""
from __future__ import annotations

import importlib

import numpy as np


def test_packaged_weights_and_envelope(tmp_path):
    L = importlib.import_module("2dfmm_gb300.learn")
    theta = L.load_weights()
    assert theta is not None and theta.dtype == np.float32 and theta.size == 10448
    k, cutoff = L.load_envelope()
    d = np.load(L.DEFAULT_WEIGHTS)
    assert cutoff == float(d["cutoff_train"]) == 3.0
    assert k == float(d["k_blobs_per_leaf_train"]) * L.ENVELOPE_FACTOR and k > 0
    # a file written without the training figure: no limit
    p = tmp_path / "w.npz"
    L.save_weights(str(p), theta, {"note": "test"})
    assert L.load_envelope(str(p)) == (0.0, 0.0)
    assert np.array_equal(L.load_weights(str(p)), theta)
    # with the figure: ENVELOPE_FACTOR times it, at the recorded radius
    L.save_weights(str(p), theta, {}, k_blobs_per_leaf_train=100.0, cutoff_train=2.5)
    assert L.load_envelope(str(p)) == (100.0 * L.ENVELOPE_FACTOR, 2.5)
