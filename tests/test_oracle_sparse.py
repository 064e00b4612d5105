"""The sparse restatement of the reference tree (oracle/tree2d_sparse.c)
against the reference's own outputs and the dense oracle, and the
extended-precision evaluation that the parity checker uses to explain
components beyond the strict per-component bar.  CPU only."""
from __future__ import annotations

import platform

import numpy as np
import pytest

from conftest import golden_names, load_golden, oracle
from test_plain_parity import assert_parity

EXACT = platform.machine() in ("x86_64", "AMD64")


@pytest.mark.parametrize("name", golden_names())
def test_sparse_tree_matches_reference(name):
    g = load_golden(name)
    s = oracle().SparseOracle(int(g["nterms"]), int(g["num_p"]), float(g["theta"]))
    s.make_tree(g["xy"], g["cir"], g["cor"])
    d = s.dump(len(g["cir"]))
    for k in ("perm", "level", "begin", "end", "leaf"):
        assert np.array_equal(d[k], g[k]), k
    for k in ("cx", "cy", "region"):
        assert np.array_equal(d[k].view(np.uint64), g[k].view(np.uint64)), k
    assert s.levels() == int(g["max_level"])
    uv = s.biot(g["txy"], threads=4)
    if EXACT:
        assert np.array_equal(uv.view(np.uint64), g["uv"].view(np.uint64))
        assert np.array_equal(d["coef"], g["coef"])
    else:
        assert np.abs(uv - g["uv"]).max() <= 1e-13 * (np.abs(g["uv"]).max() + 1e-300)


def test_sparse_equals_dense_on_a_deep_cluster():
    """About ten levels (the dense oracle still fits): the same tree,
    coefficients and velocities bit for bit, off-blob targets included."""
    O = oracle()
    rng = np.random.default_rng(3)
    xy = np.concatenate([rng.random((3000, 2)), 0.61 + 3e-3 * rng.standard_normal((1500, 2))])
    n = len(xy)
    cir = rng.standard_normal(n) / n
    cor = np.full(n, 2e-4)
    txy = np.concatenate([xy[::7], rng.random((300, 2))])
    o = O.Oracle(11, 33, 0.5)
    o.make_tree(xy, cir, cor, max_level_cap=12)
    od = o.dump(n)
    ouv = o.biot(txy, threads=4)
    levels = o.levels()
    o.close()
    s = O.SparseOracle(11, 33, 0.5)
    s.make_tree(xy, cir, cor)
    sd = s.dump(n)
    assert s.levels() == levels >= 9
    for k in ("perm", "level", "begin", "end", "leaf"):
        assert np.array_equal(sd[k], od[k]), k
    for k in ("cx", "cy", "region"):
        assert np.array_equal(sd[k].view(np.uint64), od[k].view(np.uint64)), k
    assert np.array_equal(sd["coef"], od["coef"])
    assert np.array_equal(s.biot(txy, threads=4).view(np.uint64), ouv.view(np.uint64))


@pytest.mark.parametrize("name", ["cfg1", "lamb30k", "snapshot198", "u2k"])
def test_extended_precision_value_of_the_treecode(name):
    """The reference's result differs from the extended-precision value of
    its own treecode only by FP64 rounding (normwise below 1e-13), but on a
    few cancellation components by more than 1e-12 relative: the strict
    per-component bar is out of FP64's reach there, which the parity checker
    has to know."""
    g = load_golden(name)
    s = oracle().SparseOracle(int(g["nterms"]), int(g["num_p"]), float(g["theta"]))
    s.make_tree(g["xy"], g["cir"], g["cor"])
    ext = s.biot_ext(g["txy"], threads=4)
    ref = g["uv"]
    mag = np.linalg.norm(ext, axis=1)
    assert (np.linalg.norm(ref - ext, axis=1) <= 1e-13 * mag).all()
    comp = np.abs(ref - ext) / np.maximum(np.abs(ext), 1e-300)
    misses = comp > 1e-12
    # every such component is a small fraction of its target's speed
    assert (np.abs(ext)[misses] < 0.05 * np.repeat(mag[:, None], 2, axis=1)[misses]).all()
    # the reference itself passes the checker (against itself, trivially)
    assert_parity(ref, ref, g["txy"], lambda pts: s.biot_ext(pts, cond=True), label=name)


def test_checker_catches_planted_errors():
    """Errors planted in copies of the reference's values must fail the
    checker: 1e-10 on a large component (the normwise bar), and 5e-11 on a
    component of 0.2-1.5% of its target's speed that the reference computes
    within the bar (normwise below 1e-12, so only the per-component check
    with the extended-precision value can catch it)."""
    g = load_golden("cfg1")
    s = oracle().SparseOracle(int(g["nterms"]), int(g["num_p"]), float(g["theta"]))
    s.make_tree(g["xy"], g["cir"], g["cor"])
    ref = g["uv"]
    bad = ref.copy()
    k = int(np.argmax(np.abs(ref[:, 0])))  # a large component, far from cancellation
    bad[k, 0] *= 1 + 1e-10
    with pytest.raises(AssertionError, match="normwise"):
        assert_parity(bad, ref, g["txy"], lambda pts: s.biot_ext(pts, cond=True), label="planted")
    ext = s.biot_ext(g["txy"])
    frac = np.abs(ref[:, 1]) / np.linalg.norm(ref, axis=1)
    ok = np.abs(ref[:, 1] - ext[:, 1]) <= 1e-13 * np.abs(ext[:, 1])
    k = int(np.flatnonzero((frac > 0.002) & (frac < 0.015) & ok)[0])
    bad = ref.copy()
    bad[k, 1] *= 1 + 5e-11
    with pytest.raises(AssertionError, match="not explained"):
        assert_parity(bad, ref, g["txy"], lambda pts: s.biot_ext(pts, cond=True), label="planted")
