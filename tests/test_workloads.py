"""Synthetic configurations (shapes and distributions) and the snapshot
reader/writer (the solver's s_*****_step.dat blob block)."""
from __future__ import annotations

import numpy as np

from conftest import load_golden, workloads


def test_snapshot_round_trip(tmp_path):
    W = workloads()
    rng = np.random.default_rng(0)
    xy = rng.random((37, 2))
    cir = rng.standard_normal(37)
    cor = rng.random(37) * 0.01
    p = tmp_path / "s_00001_step.dat"
    W.write_snapshot(p, xy, cir, cor)
    rxy, rcir, rcor = W.read_snapshot(p)
    assert np.array_equal(rxy, xy) and np.array_equal(rcir, cir) and np.array_equal(rcor, cor)


def test_snapshot_fixture_values_are_a_real_flow():
    g = load_golden("snapshot198")
    assert len(g["cir"]) == 27_743
    assert (g["cor"] > 0).all() and np.isfinite(g["xy"]).all()


def test_configuration_shapes():
    W = workloads()
    b = W.uniform()
    assert b.n == 20_000 and b.nterms == 11 and b.num_p == 33 and b.theta == 0.5
    assert abs(b.cir.std() * b.n - 1.0) < 0.05
    b = W.lamb_oseen(50_000)
    assert abs(b.cir.sum() - 1.0) < 1e-12 and b.nterms == 13 and b.num_p == 65
    r = np.hypot(b.xy[:, 0] - 0.5, b.xy[:, 1] - 0.5)
    assert abs(np.median(r) - 0.1 * np.sqrt(2 * np.log(2))) < 0.01  # Rayleigh(0.1) median
    b = W.two_patch_sheet(100_000)
    assert b.stored_fp32 and np.array_equal(b.xy, b.xy.astype(np.float32).astype(np.float64))
    sheet = b.cir < 0
    assert abs(sheet.mean() - 0.1) < 1e-3 and np.allclose(b.cir[sheet].sum(), -1.0, atol=1e-4)
    sets = W.batch_sets(nsets=32)
    sizes = np.array([s.n for s in sets])
    assert sizes.min() >= 2048 and sizes.max() <= 200_000
