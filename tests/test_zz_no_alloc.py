"""tree2d_solve_device_static: the solve for callers that cannot allocate GPU
memory (a host program whose device memory belongs to a pool it must not go
around, or an embedding that fixes its footprint at start-up).  It must give
the allocating entry point's answer, twice in a row on different inputs
(the shared scratch array keeps the previous call's contents), allocate
nothing, and reject inputs beyond its fixed scratch with a clear error.

Kept in its own file, named to be collected last, so that a run stopping at
the first failure has run every other test before this one.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from conftest import load_golden, workloads


def _solve_both(P, torch, b):
    dev = torch.device("cuda:0")
    xy = torch.from_numpy(np.ascontiguousarray(b["xy"])).to(dev)
    cir = torch.from_numpy(np.ascontiguousarray(b["cir"])).to(dev)
    cor = torch.from_numpy(np.ascontiguousarray(b["cor"])).to(dev)
    n = len(b["cir"])
    P.set_params(int(b["nterms"]), int(b["num_p"]), float(b["theta"]))
    ref = torch.empty((n, 2), dtype=torch.float64, device=dev)
    out = torch.full((n, 2), float("nan"), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    P.solve_device(xy.data_ptr(), cir.data_ptr(), cor.data_ptr(), ref.data_ptr(), n)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    rc = P.load().tree2d_solve_device_static(n, ctypes.c_void_p(xy.data_ptr()), ctypes.c_void_p(cir.data_ptr()),
                                             ctypes.c_void_p(cor.data_ptr()), ctypes.c_void_p(out.data_ptr()), None)
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    return rc, out.cpu().numpy(), ref.cpu().numpy(), free0 - free1


@pytest.mark.gpu
def test_static_solve_matches_allocating_solve_twice(gpu_lib):
    torch = pytest.importorskip("torch")
    P = gpu_lib
    P.set_mode(P.MODE_PLAIN)
    W = workloads()
    u = W.uniform(30_000, seed=31)
    # The first call on a device looks up the array; with lazy module loading
    # that is also when the driver places the array in device memory.
    tiny = load_golden("tiny33")
    rc, _, _, _ = _solve_both(P, torch, tiny)
    assert rc == P.OK, P.error_string(rc)
    cases = [load_golden("lamb30k"),
             dict(xy=u.xy, cir=u.cir, cor=u.cor, nterms=u.nterms, num_p=u.num_p, theta=u.theta)]
    for case in cases:  # two calls in a row, different inputs and parameters
        rc, out, ref, grew = _solve_both(P, torch, case)
        assert rc == P.OK, P.error_string(rc)
        assert np.isfinite(out).all()
        # the same kernels on the same tree: equal bit for bit, so scratch left
        # over from the previous call cannot hide behind a tolerance
        assert np.array_equal(out, ref)
        assert grew <= 0, f"device free memory fell by {grew} bytes during the call"


@pytest.mark.gpu
def test_static_solve_at_its_size_limit(gpu_lib):
    """65,536 blobs, the largest input the fixed array takes: the regions are
    sized from the tree build's own reservation, so this must fit."""
    torch = pytest.importorskip("torch")
    P = gpu_lib
    P.set_mode(P.MODE_PLAIN)
    u = workloads().uniform(P.STATIC_MAX_BLOBS, seed=32)
    case = dict(xy=u.xy, cir=u.cir, cor=u.cor, nterms=u.nterms, num_p=u.num_p, theta=u.theta)
    rc, out, ref, grew = _solve_both(P, torch, case)
    assert rc == P.OK, P.error_string(rc)
    assert np.array_equal(out, ref)
    assert grew <= 0


@pytest.mark.gpu
def test_static_solve_refuses_mixed_mode_and_mirror(gpu_lib):
    """The static solve is the plain form only: in another mode, or with a
    mirror wall, it must say so rather than answer without the images or
    with another method."""
    torch = pytest.importorskip("torch")
    P = gpu_lib
    b = load_golden("tiny33")
    dev = torch.device("cuda:0")
    xy = torch.from_numpy(np.ascontiguousarray(b["xy"])).to(dev)
    cir = torch.from_numpy(np.ascontiguousarray(b["cir"])).to(dev)
    cor = torch.from_numpy(np.ascontiguousarray(b["cor"])).to(dev)
    n = len(b["cir"])
    out = torch.full((n, 2), float("nan"), dtype=torch.float64, device=dev)
    P.set_params(int(b["nterms"]), int(b["num_p"]), float(b["theta"]))
    try:
        for mode in (P.MODE_MIXED, P.MODE_LEARNED):
            P.set_mode(mode)
            rc = P.solve_device_static(xy.data_ptr(), cir.data_ptr(), cor.data_ptr(), out.data_ptr(), n)
            assert rc == P.ERR_MODE
        P.set_mode(P.MODE_PLAIN)
        P.set_mirror(True, -0.5)
        rc = P.solve_device_static(xy.data_ptr(), cir.data_ptr(), cor.data_ptr(), out.data_ptr(), n)
        assert rc == P.ERR_MODE
        torch.cuda.synchronize()
        assert torch.isnan(out).all()  # nothing was computed
    finally:
        P.set_mirror(False, 0.0)
        P.set_mode(P.MODE_PLAIN)
    rc = P.solve_device_static(xy.data_ptr(), cir.data_ptr(), cor.data_ptr(), out.data_ptr(), n)
    assert rc == P.OK


@pytest.mark.gpu
def test_static_solve_rejects_oversize_input(gpu_lib):
    torch = pytest.importorskip("torch")
    P = gpu_lib
    P.set_params(11, 33, 0.5)
    n = P.STATIC_MAX_BLOBS + 1
    dev = torch.device("cuda:0")
    xy = torch.zeros((n, 2), dtype=torch.float64, device=dev)
    one = torch.ones(n, dtype=torch.float64, device=dev)
    out = torch.empty((n, 2), dtype=torch.float64, device=dev)
    rc = P.solve_device_static(xy.data_ptr(), one.data_ptr(), one.data_ptr(), out.data_ptr(), n)
    assert rc == P.ERR_TOO_LARGE
    assert "65536" in P.error_string(rc)
