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


def _tol_ok(a, b):
    mag = np.linalg.norm(b, axis=1, keepdims=True)
    return bool((np.abs(a - b) <= 1e-12 * np.abs(b) + 1e-13 * mag).all())


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
        assert _tol_ok(out, ref)
        assert grew <= 0, f"device free memory fell by {grew} bytes during the call"


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
