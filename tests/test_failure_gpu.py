"""Failure detection without a GPU fault.

Every wait in the library's own kernels (mbarrier waits of the tensor-core
kernels, the weight and operand bulk copies) is bounded: after a fixed
number of polls the kernel records TREE2D_ERR_TIMEOUT, drains what it has in
flight, releases its tensor memory and returns.  These tests make such a
wait run out on purpose -- a wait on a barrier that nothing completes -- and
check that the host reads the status and that the context stays usable.
"""
from __future__ import annotations

import numpy as np
import pytest


@pytest.mark.gpu
def test_bounded_wait_reports_timeout(gpu_lib):
    P = gpu_lib
    assert P.wait_probe(1000) == P.ERR_TIMEOUT
    assert P.wait_probe(200_000) == P.ERR_TIMEOUT


@pytest.mark.gpu
def test_context_usable_after_timeout(gpu_lib):
    import importlib
    P = gpu_lib
    assert P.wait_probe(5000) == P.ERR_TIMEOUT
    W = importlib.import_module("2dfmm_gb300.workloads")
    b = W.uniform(3000, seed=9)
    P.set_params(b.nterms, b.num_p, b.theta)
    for mode in (P.MODE_PLAIN, P.MODE_MIXED):
        P.set_mode(mode)
        assert P.make_tree(b.xy, b.cir, b.cor) == 0
        uv = P.biot_tree_batch(b.xy)
        assert np.isfinite(uv).all()
    P.set_mode(P.MODE_PLAIN)
