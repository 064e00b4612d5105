"""Edge cases on the GPU: empty and one-blob sets, invalid input, trees
that cannot be built, parameter override versus file."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import load_golden


@pytest.mark.gpu
def test_empty_set(gpu_lib):
    P = gpu_lib
    P.set_params(11, 33, 0.5)
    P.make_tree(np.zeros((0, 2)), np.zeros(0), np.zeros(0))
    assert P.biot_tree(0.3, 0.4) == (0.0, 0.0)


@pytest.mark.gpu
def test_non_finite_input_is_rejected(gpu_lib):
    P = gpu_lib
    P.set_params(11, 33, 0.5)
    xy = np.random.default_rng(0).random((100, 2))
    xy[17, 0] = np.nan
    rc = P.make_tree(xy, np.ones(100), np.ones(100), check=False)
    assert rc == P.ERR_BAD_INPUT
    u, v = P.biot_tree(0.5, 0.5)
    assert np.isnan(u) and np.isnan(v)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["plain", "mixed"])
@pytest.mark.parametrize("field,value", [("cir", np.inf), ("cir", np.nan), ("cor", np.nan)])
def test_non_finite_circulation_or_core_is_rejected(gpu_lib, mode, field, value):
    """Circulations and core radii are uploaded beside the tree build and
    checked where the build first reads them: a bad value still fails the
    make_tree call, and the next valid call succeeds."""
    P = gpu_lib
    P.set_params(11, 33, 0.5)
    P.set_mode(P.MODE_PLAIN if mode == "plain" else P.MODE_MIXED)
    try:
        rng = np.random.default_rng(2)
        xy = rng.random((5000, 2))
        cir = rng.standard_normal(5000) / 5000
        cor = np.full(5000, 0.01)
        bad = {"cir": cir.copy(), "cor": cor.copy()}
        bad[field][1234] = value
        rc = P.make_tree(xy, bad["cir"], bad["cor"], check=False)
        assert rc == P.ERR_BAD_INPUT
        assert P.make_tree(xy, cir, cor, check=False) == 0
        uv = P.biot_tree_batch(xy)
        assert np.isfinite(uv).all()
    finally:
        P.set_mode(P.MODE_PLAIN)


@pytest.mark.gpu
def test_too_many_coincident_blobs(gpu_lib):
    """num_p blobs at one point can never be separated: the reference grows
    its max level forever; the library reports TREE2D_ERR_TOO_DEEP."""
    P = gpu_lib
    P.set_params(11, 33, 0.5)
    xy = np.random.default_rng(1).random((200, 2))
    xy[:40] = xy[0]
    rc = P.make_tree(xy, np.ones(200), np.ones(200), check=False)
    assert rc == P.ERR_TOO_DEEP
    # a valid call afterwards works again
    g = load_golden("u2k")
    P.make_tree(g["xy"], g["cir"], g["cor"])
    assert np.isfinite(P.biot_tree(0.5, 0.5)).all()


@pytest.mark.gpu
def test_tiny_sets_and_leaf_threshold(gpu_lib):
    P = gpu_lib
    for name in ("tiny1", "tiny2", "tiny32", "tiny33"):
        g = load_golden(name)
        P.set_params(int(g["nterms"]), int(g["num_p"]), float(g["theta"]))
        P.make_tree(g["xy"], g["cir"], g["cor"])
        uv = P.biot_tree_batch(g["txy"])
        assert np.allclose(uv, g["uv"], rtol=1e-12, atol=1e-300), name


@pytest.mark.gpu
def test_param_file_drives_make_tree(gpu_lib, tmp_path, monkeypatch):
    P = gpu_lib
    g = load_golden("u2k")
    (tmp_path / "cal_cond").mkdir()
    (tmp_path / "run").mkdir()
    (tmp_path / "cal_cond" / "fmm_param.dat").write_text(
        f"{int(g['nterms'])}    nterms\n{int(g['num_p'])}   num_p\n{float(g['theta'])}d0 theta\n0.01  r_min ! for Tree\n")
    monkeypatch.chdir(tmp_path / "run")
    P.clear_params()
    P.make_tree(g["xy"], g["cir"], g["cor"])
    uv = P.biot_tree_batch(g["txy"])
    assert np.abs(uv - g["uv"]).max() <= 1e-12 * np.abs(g["uv"]).max()


@pytest.mark.gpu
def test_mirror_wall_against_direct_sum_with_images(gpu_lib):
    """A wall at y = d: images (x, 2d - y) with -G as point vortices."""
    from conftest import oracle
    P = gpu_lib
    rng = np.random.default_rng(5)
    xy = rng.random((3000, 2)) * [1.0, 0.5] + [0.0, 0.1]
    cir = rng.standard_normal(3000) / 3000
    cor = np.full(3000, 0.01)
    d = 0.05
    sxy = np.concatenate([xy, np.stack([xy[:, 0], 2 * d - xy[:, 1]], 1)])
    ref = oracle().direct(xy, sxy, np.concatenate([cir, -cir]), np.concatenate([cor, np.zeros(3000)]))
    P.set_params(11, 33, 0.5)
    P.set_mirror(True, d)
    try:
        for mode, tol in ((P.MODE_PLAIN, 5e-6), (P.MODE_MIXED, 1e-6)):
            P.set_mode(mode)
            P.make_tree(xy, cir, cor)
            uv = P.biot_tree_batch(xy)
            assert np.linalg.norm(uv - ref) / np.linalg.norm(ref) <= tol, mode
    finally:
        P.set_mirror(False)
        P.set_mode(P.MODE_PLAIN)


@pytest.mark.gpu
def test_advect_device(gpu_lib):
    torch = pytest.importorskip("torch")
    P = gpu_lib
    dev = torch.device("cuda:0")
    xy = torch.rand((1000, 2), dtype=torch.float64, device=dev)
    uv = torch.randn((1000, 2), dtype=torch.float64, device=dev)
    ref = xy + 1e-3 * uv
    P.advect_device(xy.data_ptr(), uv.data_ptr(), 1000, 1e-3)
    torch.cuda.synchronize()
    assert torch.equal(xy, ref)
