"""FP64 direct-sum kernel (the accuracy yardstick) against the oracle's direct sum."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import oracle


@pytest.mark.gpu
def test_direct_kernel_matches_oracle(gpu_lib):
    torch = pytest.importorskip("torch")
    P = gpu_lib
    rng = np.random.default_rng(3)
    sxy = rng.random((5000, 2))
    cir = rng.standard_normal(5000) / 5000
    cor = np.full(5000, 0.01)
    txy = np.concatenate([sxy[:100], rng.random((300, 2))])
    ref = oracle().direct(txy, sxy, cir, cor)
    dev = torch.device("cuda:0")
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)  # noqa: E731
    out = torch.empty((len(txy), 2), dtype=torch.float64, device=dev)
    tt, ss, cc, rr = t(txy), t(sxy), t(cir), t(cor)
    P.direct_device(tt.data_ptr(), len(txy), ss.data_ptr(), cc.data_ptr(), rr.data_ptr(), len(cir), out.data_ptr())
    torch.cuda.synchronize()
    uv = out.cpu().numpy()
    assert np.abs(uv - ref).max() <= 1e-12 * np.abs(ref).max()
