"""The oracle against the reference itself on seeded random inputs, beyond
the committed goldens: the reference built from its own sources
(oracle/_ref/ref_driver, ver-c/src unmodified) runs in a fresh process on
each case, and the oracle must reproduce its tree (permutation, levels,
ranges, leaf flags, centres, sides) bit for bit and its velocities bit for
bit on x86-64 (within 1e-13 of the largest speed elsewhere, where libm's cpow
may round differently).  Parameters vary over the ranges the reference's
parameter file takes (nterms, num_p, theta), and so do the distributions:
uniform, a tight cluster with coincident blobs, and a thin sheet.  Skipped
where the reference's sources were not available to build it."""
from __future__ import annotations

import platform

import numpy as np
import pytest

from conftest import oracle

EXACT = platform.machine() in ("x86_64", "AMD64")

CASES = [
    # seed, n, nterms, num_p, theta, distribution
    (101, 1500, 11, 33, 0.5, "uniform"),
    (102, 2500, 5, 9, 0.3, "uniform"),
    (103, 1200, 17, 17, 0.8, "cluster"),
    (104, 3000, 13, 65, 0.5, "sheet"),
    # num_p above the 9 coincident blobs: with num_p <= 9 they never split
    # and the reference itself crashes (the library reports TREE2D_ERR_TOO_DEEP)
    (105, 800, 2, 12, 0.6, "cluster"),
    (106, 2000, 21, 40, 0.45, "sheet"),
]


def make_case(seed, n, kind):
    rng = np.random.default_rng(seed)
    if kind == "uniform":
        xy = rng.uniform(0.0, 1.0, (n, 2))
    elif kind == "cluster":
        xy = 0.5 + 1e-3 * rng.standard_normal((n, 2))
        xy[n // 2: n // 2 + 8] = xy[0]  # coincident blobs
    else:
        x = rng.uniform(0.0, 1.0, n)
        xy = np.stack([x, 0.2 + 0.01 * np.sin(8 * np.pi * x) + 1e-5 * rng.standard_normal(n)], axis=1)
    cir = rng.standard_normal(n) / n
    cor = np.full(n, 0.5 / np.sqrt(n))
    off = rng.uniform(0.0, 1.0, (64, 2))  # points that are not blobs
    txy = np.concatenate([xy, off])
    return xy, cir, cor, txy


@pytest.mark.parametrize("case", CASES, ids=[f"{c[5]}-{c[1]}-p{c[2]}-n{c[3]}-t{c[4]}" for c in CASES])
def test_oracle_matches_reference_build(case, tmp_path):
    O = oracle()
    if not O.reference_available():
        pytest.skip("the reference's own build is not available here")
    seed, n, nterms, num_p, theta, kind = case
    xy, cir, cor, txy = make_case(seed, n, kind)
    ref = O.run_reference(str(tmp_path), xy, cir, cor, txy, nterms, num_p, theta)
    o = O.Oracle(nterms, num_p, theta)
    o.make_tree(xy, cir, cor)
    uv = o.biot(txy, threads=2)
    d = o.dump(n)
    for k in ("perm", "level", "begin", "end", "leaf"):
        assert np.array_equal(d[k], ref[k]), k
    for k in ("cx", "cy", "region"):
        assert np.array_equal(d[k].view(np.uint64), ref[k].view(np.uint64)), k
    assert o.levels() == ref["max_level"]
    if EXACT:
        assert np.array_equal(uv.view(np.uint64), ref["uv"].view(np.uint64))
    else:
        assert np.abs(uv - ref["uv"]).max() <= 1e-13 * (np.abs(ref["uv"]).max() + 1e-300)
