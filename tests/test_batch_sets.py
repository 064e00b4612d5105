"""Batched solve of independent blob sets in one tree (configuration 4's
form): every set's velocities must equal solving that set by itself, bit
for bit, and meet the mixed form's accuracy against the FP64 direct sum."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import workloads


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).to(torch.device("cuda:0"))


def _concat(sets):
    xy = np.concatenate([b.xy for b in sets])
    cir = np.concatenate([b.cir for b in sets])
    cor = np.concatenate([b.cor for b in sets])
    off = np.concatenate([[0], np.cumsum([b.n for b in sets])]).astype(np.int32)
    return xy, cir, cor, off


@pytest.mark.gpu
def test_batched_sets_equal_single_solves(gpu_lib):
    torch = pytest.importorskip("torch")
    P = gpu_lib
    W = workloads()
    sets = W.batch_sets(nsets=7, seed=41, lo=2048, hi=30_000)
    b0 = sets[0]
    P.set_params(b0.nterms, b0.num_p, b0.theta)
    P.set_mode(P.MODE_MIXED)
    P.set_mixed_params(16, 3.0, True)
    xy, cir, cor, off = _concat(sets)
    d_xy, d_cir, d_cor = _dev(torch, xy), _dev(torch, cir), _dev(torch, cor)
    d_uv = torch.empty_like(d_xy)
    torch.cuda.synchronize()
    P.solve_sets(d_xy.data_ptr(), d_cir.data_ptr(), d_cor.data_ptr(), d_uv.data_ptr(), off)
    torch.cuda.synchronize()
    st = P.stats()
    assert st["n_blobs"] == off[-1]
    uv = d_uv.cpu().numpy()
    for k, b in enumerate(sets):
        s_xy, s_cir, s_cor = _dev(torch, b.xy), _dev(torch, b.cir), _dev(torch, b.cor)
        s_uv = torch.empty_like(s_xy)
        P.solve_device(s_xy.data_ptr(), s_cir.data_ptr(), s_cor.data_ptr(), s_uv.data_ptr(), b.n)
        torch.cuda.synchronize()
        assert np.array_equal(uv[off[k]:off[k + 1]], s_uv.cpu().numpy()), f"set {k} (n={b.n})"
    # accuracy of two sets against the FP64 direct sum
    for k in (0, len(sets) - 1):
        b = sets[k]
        idx = W.sample_targets(b.n, 512, seed=k)
        s_xy, s_cir, s_cor = _dev(torch, b.xy), _dev(torch, b.cir), _dev(torch, b.cor)
        txy = s_xy[torch.from_numpy(idx).to(s_xy.device)].contiguous()
        ref = torch.empty_like(txy)
        P.direct_device(txy.data_ptr(), len(idx), s_xy.data_ptr(), s_cir.data_ptr(), s_cor.data_ptr(), b.n,
                        ref.data_ptr())
        torch.cuda.synchronize()
        got = uv[off[k]:off[k + 1]][idx]
        ref = ref.cpu().numpy()
        assert np.linalg.norm(got - ref) / np.linalg.norm(ref) <= 1e-6
    P.set_mode(P.MODE_PLAIN)


@pytest.mark.gpu
def test_batched_sets_learned_equal_single_solves(gpu_lib):
    """The learned mode on a batched tree: each set's decisions use its own
    reference scale u_ref (the one it has alone), so every set's velocities
    equal its learned solve alone, bit for bit; the network skips work on
    the sets with weak sources (the sheets), and the batch keeps relL2 <=
    1e-6."""
    torch = pytest.importorskip("torch")
    import importlib
    P = gpu_lib
    W = workloads()
    L = importlib.import_module("2dfmm_gb300.learn")
    theta = L.load_weights()
    if theta is None:
        pytest.skip("no packaged weights")
    sets = [W.two_patch_sheet(n, seed=50 + k) for k, n in enumerate((24_000, 41_000, 60_000))]
    sets += W.batch_sets(nsets=3, seed=43, lo=4096, hi=30_000)
    b0 = sets[0]
    P.set_params(b0.nterms, b0.num_p, b0.theta)
    P.set_mixed_params(16, 2.5, True)
    P.learn_set_weights(theta)
    P.learn_set_options(1.0, 1)
    P.learn_set_envelope(*L.load_envelope())
    xy, cir, cor, off = _concat(sets)
    d_xy, d_cir, d_cor = _dev(torch, xy), _dev(torch, cir), _dev(torch, cor)
    try:
        pairs = {}
        for mode in (P.MODE_MIXED, P.MODE_LEARNED):
            P.set_mode(mode)
            d_uv = torch.empty_like(d_xy)
            P.solve_sets(d_xy.data_ptr(), d_cir.data_ptr(), d_cor.data_ptr(), d_uv.data_ptr(), off)
            torch.cuda.synchronize()
            pairs[mode] = P.stats()["n_pairs"]
        assert P.stats()["learned_active"] == 1
        assert pairs[P.MODE_LEARNED] < pairs[P.MODE_MIXED]
        uv = d_uv.cpu().numpy()
        assert np.all(np.isfinite(uv))
        for k, b in enumerate(sets):
            s_xy, s_cir, s_cor = _dev(torch, b.xy), _dev(torch, b.cir), _dev(torch, b.cor)
            s_uv = torch.empty_like(s_xy)
            P.solve_device(s_xy.data_ptr(), s_cir.data_ptr(), s_cor.data_ptr(), s_uv.data_ptr(), b.n)
            torch.cuda.synchronize()
            assert P.stats()["learned_active"] == 1
            assert np.array_equal(uv[off[k]:off[k + 1]], s_uv.cpu().numpy()), f"set {k} (n={b.n})"
            # 4,096 sampled targets per set, as configuration 4 measures
            # (with 512 the estimate of a 24k-blob set's relL2 moved by 40%)
            idx = W.sample_targets(b.n, 4096, seed=k)
            txy = s_xy[torch.from_numpy(idx).to(s_xy.device)].contiguous()
            ref = torch.empty_like(txy)
            P.direct_device(txy.data_ptr(), len(idx), s_xy.data_ptr(), s_cir.data_ptr(), s_cor.data_ptr(), b.n,
                            ref.data_ptr())
            torch.cuda.synchronize()
            ref = ref.cpu().numpy()
            got = uv[off[k]:off[k + 1]][idx]
            assert np.linalg.norm(got - ref) / np.linalg.norm(ref) <= 1e-6, f"set {k}"
    finally:
        P.set_mode(P.MODE_PLAIN)


@pytest.mark.gpu
def test_batched_sets_reject_plain_mode_and_bad_offsets(gpu_lib):
    torch = pytest.importorskip("torch")
    P = gpu_lib
    W = workloads()
    sets = W.batch_sets(nsets=2, seed=5, lo=2048, hi=4096)
    xy, cir, cor, off = _concat(sets)
    d_xy, d_cir, d_cor = _dev(torch, xy), _dev(torch, cir), _dev(torch, cor)
    d_uv = torch.empty_like(d_xy)
    P.set_params(sets[0].nterms, sets[0].num_p, sets[0].theta)
    P.set_mode(P.MODE_PLAIN)
    with pytest.raises(RuntimeError):
        P.solve_sets(d_xy.data_ptr(), d_cir.data_ptr(), d_cor.data_ptr(), d_uv.data_ptr(), off)
    assert P.last_error() == P.ERR_MODE
    P.set_mode(P.MODE_MIXED)
    bad = off.copy()
    bad[1] = bad[2] + 1  # decreasing
    with pytest.raises(RuntimeError):
        P.solve_sets(d_xy.data_ptr(), d_cir.data_ptr(), d_cor.data_ptr(), d_uv.data_ptr(), bad)
    assert P.last_error() == P.ERR_BAD_INPUT
    P.set_mode(P.MODE_PLAIN)


@pytest.mark.gpu
def test_batched_sets_with_empty_and_tiny_sets(gpu_lib):
    """Empty sets and one-blob sets in the batch: the others are unchanged."""
    torch = pytest.importorskip("torch")
    P = gpu_lib
    W = workloads()
    big = W.batch_sets(nsets=2, seed=77, lo=3000, hi=6000)
    one = W.batch_sets(nsets=1, seed=78, lo=2048, hi=2048)[0]
    one.xy, one.cir, one.cor = one.xy[:1], one.cir[:1], one.cor[:1]
    empty = W.batch_sets(nsets=1, seed=79, lo=2048, hi=2048)[0]
    empty.xy, empty.cir, empty.cor = empty.xy[:0], empty.cir[:0], empty.cor[:0]
    sets = [big[0], empty, one, big[1], empty]
    P.set_params(big[0].nterms, big[0].num_p, big[0].theta)
    P.set_mode(P.MODE_MIXED)
    P.set_mixed_params(16, 3.0, True)
    xy, cir, cor, off = _concat(sets)
    d_xy, d_cir, d_cor = _dev(torch, xy), _dev(torch, cir), _dev(torch, cor)
    d_uv = torch.empty_like(d_xy)
    P.solve_sets(d_xy.data_ptr(), d_cir.data_ptr(), d_cor.data_ptr(), d_uv.data_ptr(), off)
    torch.cuda.synchronize()
    uv = d_uv.cpu().numpy()
    assert np.all(uv[off[2]:off[3]] == 0.0)  # a lone blob induces nothing on itself
    for k in (0, 3):
        b = sets[k]
        s_xy, s_cir, s_cor = _dev(torch, b.xy), _dev(torch, b.cir), _dev(torch, b.cor)
        s_uv = torch.empty_like(s_xy)
        P.solve_device(s_xy.data_ptr(), s_cir.data_ptr(), s_cor.data_ptr(), s_uv.data_ptr(), b.n)
        torch.cuda.synchronize()
        assert np.array_equal(uv[off[k]:off[k + 1]], s_uv.cpu().numpy())
    P.set_mode(P.MODE_PLAIN)
