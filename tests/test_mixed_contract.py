"""The accuracy contract of the approximate modes (TREE2D_MODE_MIXED and
TREE2D_MODE_LEARNED) for every query they answer, at the shipped defaults
(correction radius 2.5 max sigma, leaf size by set size, the packaged
network): relL2 <= 1e-6 against the FP64 direct sum at blob positions and at
points that are not blobs (the solver's sheet centres, e_velo_mpi.f90:59-64,
are such points), with the max relative error reported beside it."""
from __future__ import annotations

import importlib

import numpy as np
import pytest

from conftest import workloads

REL_L2 = 1e-6


def _defaults(P, mode):
    P.set_mode(mode)
    P.set_mixed_params(16, 2.5, True)
    P.set_mixed_leaf(-1)
    P.set_tuning(True, -1)
    if mode == P.MODE_LEARNED:
        L = importlib.import_module("2dfmm_gb300.learn")
        theta = L.load_weights()
        assert theta is not None, "packaged weights missing"
        P.learn_set_weights(theta)
        P.learn_set_options(1.0, 1)
        P.learn_set_envelope(*L.load_envelope())


def _direct(P, torch, b, pts):
    dev = torch.device("cuda:0")
    sxy = torch.from_numpy(b.xy).to(dev)
    cir = torch.from_numpy(b.cir).to(dev)
    cor = torch.from_numpy(b.cor).to(dev)
    txy = torch.from_numpy(np.ascontiguousarray(pts)).to(dev)
    out = torch.empty_like(txy)
    P.direct_device(txy.data_ptr(), len(pts), sxy.data_ptr(), cir.data_ptr(), cor.data_ptr(), b.n, out.data_ptr())
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _errors(got, ref):
    rel = float(np.linalg.norm(got - ref) / np.linalg.norm(ref))
    mx = float((np.linalg.norm(got - ref, axis=1) / np.maximum(np.linalg.norm(ref, axis=1), 1e-300)).max())
    return rel, mx


def _off_blob_points(b, rng, k=4096):
    """Sheet centres (midpoints of neighbouring sheet blobs along x), points
    scattered over and around the patches, points just off blobs, and points
    outside the root box."""
    ns = int(b.n - 2 * round(0.45 * b.n))
    sheet = b.xy[b.n - ns:]
    sheet = sheet[np.argsort(sheet[:, 0])]
    mid = 0.5 * (sheet[1:] + sheet[:-1])
    mid = mid[rng.choice(len(mid), k, replace=False)]
    scatter = np.column_stack([rng.uniform(0.2, 0.8, k), rng.uniform(0.15, 0.85, k)])
    near = b.xy[rng.choice(b.n, k // 4, replace=False)] + 1e-6 * rng.standard_normal((k // 4, 2))
    outside = np.array([[-0.5, 0.5], [1.5, 0.5], [0.5, -1.0], [0.5, 3.0], [-2.0, -2.0], [4.0, 4.0]])
    return {"sheet centres": mid, "scattered": scatter, "just off blobs": near, "outside the root box": outside}


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["mixed", "learned"])
def test_off_blob_points_keep_the_mixed_accuracy(gpu_lib, mode):
    """Points that are not blob positions are answered by a traversal of the
    mixed tree (far cells by their multipoles, the rest pair by pair), not by
    the plain treecode (relL2 ~4e-4 on such sets): relL2 <= 1e-6 for each
    kind of point, and single biot_tree calls equal the batch answers."""
    torch = pytest.importorskip("torch")
    P = gpu_lib
    W = workloads()
    b = W.two_patch_sheet(524_288, seed=23)
    P.set_params(b.nterms, b.num_p, b.theta)
    _defaults(P, P.MODE_MIXED if mode == "mixed" else P.MODE_LEARNED)
    try:
        P.make_tree(b.xy, b.cir, b.cor)
        rng = np.random.default_rng(41)
        kinds = _off_blob_points(b, rng)
        pts = np.concatenate(list(kinds.values()))
        uv = P.biot_tree_batch(pts)
        ref = _direct(P, torch, b, pts)
        o = 0
        report = []
        for name, k in kinds.items():
            rel, mx = _errors(uv[o:o + len(k)], ref[o:o + len(k)])
            report.append(f"{name}: relL2 {rel:.2e}, max rel {mx:.2e}")
            assert rel <= REL_L2, f"{mode} {name}: relL2 {rel:.3e}"
            o += len(k)
        print(f"[off-blob] {mode}: " + "; ".join(report))
        for i in (0, 1, len(pts) // 2, len(pts) - 1):
            u, v = P.biot_tree(*pts[i])
            assert u == uv[i, 0] and v == uv[i, 1]
    finally:
        P.set_mode(P.MODE_PLAIN)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["mixed", "learned"])
def test_shipped_defaults_keep_accuracy(gpu_lib, mode):
    """The shipped configuration (radius 2.5, default leaf size, packaged
    weights) on the two-patch + sheet distribution at 1/8 size, 4,096
    sampled blob targets."""
    torch = pytest.importorskip("torch")
    P = gpu_lib
    W = workloads()
    b = W.two_patch_sheet(524_288, seed=3)
    P.set_params(b.nterms, b.num_p, b.theta)
    _defaults(P, P.MODE_MIXED if mode == "mixed" else P.MODE_LEARNED)
    dev = torch.device("cuda:0")
    try:
        xy = torch.from_numpy(b.xy).to(dev)
        cir = torch.from_numpy(b.cir).to(dev)
        cor = torch.from_numpy(b.cor).to(dev)
        uv = torch.empty_like(xy)
        P.solve_device(xy.data_ptr(), cir.data_ptr(), cor.data_ptr(), uv.data_ptr(), b.n)
        torch.cuda.synchronize()
        idx = W.sample_targets(b.n, 4096, seed=8)
        rel, mx = _errors(uv.cpu().numpy()[idx], _direct(P, torch, b, b.xy[idx]))
        print(f"[defaults] {mode} 524,288 blobs: relL2 {rel:.2e}, max rel {mx:.2e}")
        assert rel <= REL_L2, rel
    finally:
        P.set_mode(P.MODE_PLAIN)


@pytest.mark.gpu
def test_shipped_defaults_full_configuration_3(gpu_lib):
    """Configuration 3 in full (4,194,304 blobs) with every default and the
    packaged network, measured on 65,536 seeded targets as the benchmark
    measures it; the network's decisions must be in force."""
    torch = pytest.importorskip("torch")
    P = gpu_lib
    W = workloads()
    b = W.two_patch_sheet()
    P.set_params(b.nterms, b.num_p, b.theta)
    _defaults(P, P.MODE_LEARNED)
    dev = torch.device("cuda:0")
    try:
        xy = torch.from_numpy(b.xy).to(dev)
        cir = torch.from_numpy(b.cir).to(dev)
        cor = torch.from_numpy(b.cor).to(dev)
        uv = torch.empty_like(xy)
        P.solve_device(xy.data_ptr(), cir.data_ptr(), cor.data_ptr(), uv.data_ptr(), b.n)
        torch.cuda.synchronize()
        st = P.stats()
        idx = W.sample_targets(b.n, 65_536, seed=7)
        rel, mx = _errors(uv.cpu().numpy()[idx], _direct(P, torch, b, b.xy[idx]))
        print(f"[defaults] learned 4,194,304 blobs: relL2 {rel:.2e}, max rel {mx:.2e}, "
              f"learned_active {st['learned_active']}, pairs/target {st['n_pairs'] / b.n:.0f}")
        assert st["learned_active"] == 1
        assert rel <= REL_L2, rel
    finally:
        P.set_mode(P.MODE_PLAIN)
