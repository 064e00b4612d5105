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
    assert cutoff == float(d["cutoff_train"]) == L.TRAIN_CUTOFF
    assert k == float(d["k_blobs_per_leaf_train"]) * L.ENVELOPE_FACTOR and k > 0
    # a file written without the training figure: no limit
    p = tmp_path / "w.npz"
    L.save_weights(str(p), theta, {"note": "test"})
    assert L.load_envelope(str(p)) == (0.0, 0.0)
    assert np.array_equal(L.load_weights(str(p)), theta)
    # with the figure: ENVELOPE_FACTOR times it, at the recorded radius
    L.save_weights(str(p), theta, {}, k_blobs_per_leaf_train=100.0, cutoff_train=2.5)
    assert L.load_envelope(str(p)) == (100.0 * L.ENVELOPE_FACTOR, 2.5)


def test_raw_weights_file_loads_through_the_c_abi(lib, tmp_path):
    """The packaged .t2dw file is the .npz's network and envelope, and the C
    loader (the way C and Fortran callers enable the learned mode) sets
    exactly those; a malformed or missing file changes nothing."""
    import ctypes
    P = importlib.import_module("2dfmm_gb300")
    L = importlib.import_module("2dfmm_gb300.learn")
    theta = L.load_weights()
    raw = open(L.DEFAULT_RAW_WEIGHTS, "rb").read()
    assert raw[:4] == b"T2DW"
    assert np.array_equal(np.frombuffer(raw[32:], "<f4"), theta)
    assert np.frombuffer(raw[16:32], "<f8").tolist() == list(L.load_envelope())
    assert P.learn_load(L.DEFAULT_RAW_WEIGHTS) == P.OK
    assert np.array_equal(P.learn_get_weights(), theta)
    # a file for another network size, a truncated file, a missing file
    bad = tmp_path / "bad.t2dw"
    L.write_raw_weights(str(bad), np.ones(17, np.float32))
    assert P.learn_load(str(bad)) == P.ERR_FILE
    bad.write_bytes(raw[:1000])
    assert P.learn_load(str(bad)) == P.ERR_FILE
    assert P.learn_load(str(tmp_path / "none.t2dw")) == P.ERR_FILE
    assert np.array_equal(P.learn_get_weights(), theta)
    assert "weights file" in P.error_string(P.ERR_FILE)
    # saving a network writes both files
    p = tmp_path / "w.npz"
    L.save_weights(str(p), theta * 2, {}, k_blobs_per_leaf_train=10.0, cutoff_train=2.5)
    assert P.learn_load(str(tmp_path / "w.t2dw")) == P.OK
    assert np.array_equal(P.learn_get_weights(), theta * 2)
    assert ctypes.sizeof(P.Stats) > 0
