"""The oracle against the reference's own outputs (golden vectors made by
running the reference built from its sources; tests/golden/make_golden.py),
and known-answer tests of the index algebra (ver-c/src/morton_order.c:4-51,
ver-c/src/quadtree.c:29-35)."""
from __future__ import annotations

import platform

import numpy as np
import pytest

from conftest import golden_names, load_golden, oracle

# Goldens were produced on x86-64; the oracle there is bit-exact.  On other
# platforms libm's cpow/exp may round differently in the last place.
EXACT = platform.machine() in ("x86_64", "AMD64")


@pytest.mark.parametrize("name", golden_names())
def test_oracle_matches_reference(name):
    O = oracle()
    g = load_golden(name)
    o = O.Oracle(int(g["nterms"]), int(g["num_p"]), float(g["theta"]))
    o.make_tree(g["xy"], g["cir"], g["cor"])
    uv = o.biot(g["txy"], threads=4)
    d = o.dump(len(g["cir"]))
    for k in ("perm", "level", "begin", "end", "leaf"):
        assert np.array_equal(d[k], g[k]), k
    for k in ("cx", "cy", "region"):
        assert np.array_equal(d[k].view(np.uint64), g[k].view(np.uint64)), k
    if EXACT:
        assert np.array_equal(uv.view(np.uint64), g["uv"].view(np.uint64))
        assert np.array_equal(d["coef"], g["coef"])
    else:
        scale = np.abs(g["uv"]).max() + 1e-300
        assert np.abs(uv - g["uv"]).max() <= 1e-13 * scale
    assert o.levels() == int(g["max_level"])


def test_oracle_direct_matches_leafwise_formula():
    O = oracle()
    rng = np.random.default_rng(0)
    sxy = rng.random((300, 2))
    cir = rng.standard_normal(300)
    cor = np.full(300, 0.05)
    txy = np.concatenate([sxy[:10], rng.random((10, 2))])
    uv = O.direct(txy, sxy, cir, cor, threads=1)
    # independent numpy restatement of the pair kernel (fmm.c:121-142)
    rx = txy[:, None, 0] - sxy[None, :, 0]
    ry = txy[:, None, 1] - sxy[None, :, 1]
    r = np.sqrt(rx * rx + ry * ry)
    with np.errstate(divide="ignore", invalid="ignore"):
        rv = np.where(r > 1e-10, cir * (1 - np.exp(-(r / cor) ** 2)) / (r * r), 0.0)
    ref = np.stack([-(rv * ry).sum(1), (rv * rx).sum(1)], 1) * 0.5 / np.pi
    assert np.allclose(uv, ref, rtol=1e-12, atol=1e-14 * np.abs(ref).max())


def test_index_algebra_known_answers():
    L = oracle().lib()
    import ctypes
    L.ora_child.restype = ctypes.c_long
    L.ora_child.argtypes = [ctypes.c_long, ctypes.c_int]
    L.ora_parent.restype = ctypes.c_long
    L.ora_parent.argtypes = [ctypes.c_long]
    L.ora_level_of.argtypes = [ctypes.c_long]
    L.ora_global2local.restype = ctypes.c_long
    L.ora_global2local.argtypes = [ctypes.c_long, ctypes.c_int]
    L.ora_quadrant.argtypes = [ctypes.c_double] * 4
    assert [L.ora_child(3, q) for q in range(4)] == [13, 14, 15, 16]   # slide 7 of the reference deck
    assert [L.ora_child(2, q) for q in range(4)] == [9, 10, 11, 12]
    assert L.ora_parent(19) == 4
    assert L.ora_level_of(13) == 2
    assert L.ora_global2local(13, 2) == 8
    assert L.ora_quadrant(1.0, -1.0, 0.0, 0.0) == 3
    # ties: x == cx counts as the + side, y == cy as the - side
    assert L.ora_quadrant(0.0, 0.0, 0.0, 0.0) == 3
    assert L.ora_quadrant(-1.0, 1.0, 0.0, 0.0) == 0


def test_param_file_quirk(tmp_path):
    """The shipped parameter file uses a Fortran literal (0.5d0): the
    reference's fscanf stops at 'd', so theta = 0.5 and r_min is not read."""
    O = oracle()
    L = O.lib()
    cc = tmp_path / "cal_cond"
    cc.mkdir()
    (cc / "fmm_param.dat").write_text("15    nterms\n250   num_p\n0.5d0 theta\n0.01  r_min ! for Tree\n")
    xy = np.random.default_rng(1).random((50, 2))
    O.Oracle(11, 33, 0.7)  # parameters before the file is read
    import ctypes
    rc = L.ora_make_tree(50, xy.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                         np.ones(50).ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                         np.ones(50).ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                         str(cc / "fmm_param.dat").encode(), 20)
    assert rc == 0
    assert L.ora_nterms() == 15 and L.ora_num_p() == 250
    L.ora_theta.restype = ctypes.c_double
    assert L.ora_theta() == 0.5
