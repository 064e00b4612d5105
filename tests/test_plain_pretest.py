"""The plain kernel's FP32 opening pre-test (k_eval in 2dfmm_gb300/csrc/plain.cu)
must never decide differently from the FP64 test it stands in front of.

The rule, restated here in numpy float32 with the kernel's roundings: the
target and the cell centre as FP32 pairs (hi = nearest float, lo = the rest
rounded), dxf = (xh - cxh) + (xl - cxl), d2f = fma(dxf, dxf, dyf * dyf),
err = fma(2^-20, d2f, ef (|dxf| + |dyf| + ef)) with ef = 2^-44 (|xh| + |yh|
+ |cxh| + |cyh|); d2f + err (rounded up) below the lower bound rounded down
to FP32 opens the cell, d2f - err (rounded down) above the upper bound
rounded up accepts it, anything else takes the FP64 test.  The FP64 test is
the reference's (quadtree/fmm.c:69-118: region > theta * sqrt(d2)) behind the
per-cell bounds region^2 / (theta^2 (1 +- 2e-13)).

Pairs are placed near the opening boundary (relative offsets 1e-12..1e-1), over
coordinate scales 1e-6..1e6, cell levels 1..32 and centres far from the
origin relative to the cell (the cancellation case)."""
import numpy as np

F = np.float32


def _round_dir(v64, f, up):
    """f (float32 nearest of v64) moved one ulp outwards where it fell on the wrong side."""
    if up:
        return np.where(f.astype(np.float64) < v64, np.nextafter(f, F(np.inf)), f)
    return np.where(f.astype(np.float64) > v64, np.nextafter(f, F(-np.inf)), f)


def _split(v):
    h = v.astype(F)
    return h, (v - h.astype(np.float64)).astype(F)


def _pretest(x, y, cx, cy, mbx, mby):
    """(sure_open, sure_accept) of the FP32 pre-test."""
    xh, xl = _split(x)
    yh, yl = _split(y)
    cxh, cxl = _split(cx)
    cyh, cyl = _split(cy)
    lo = np.where(mbx >= 1e-30, _round_dir(mbx, mbx.astype(F), False), F(-1))
    hi = np.where(mby >= 1e-30, _round_dir(mby, mby.astype(F), True), F(np.inf))
    with np.errstate(all="ignore"):
        dxf = (xh - cxh) + (xl - cxl)
        dyf = (yh - cyh) + (yl - cyl)
        # one rounding for the fma: the float64 sum of a float32 square and a
        # float32 product is exact enough for these magnitudes
        d2f = (dxf.astype(np.float64) ** 2 + (dyf * dyf).astype(np.float64)).astype(F)
        ef = F(2.0 ** -44) * ((np.abs(xh) + np.abs(yh)) + (np.abs(cxh) + np.abs(cyh)))
        err = (F(2.0 ** -20) * d2f.astype(np.float64)
               + (ef * ((np.abs(dxf) + np.abs(dyf)) + ef)).astype(np.float64)).astype(F)
        up = d2f.astype(np.float64) + err.astype(np.float64)
        dn = d2f.astype(np.float64) - err.astype(np.float64)
        s_up = _round_dir(up, up.astype(F), True)
        s_dn = _round_dir(dn, dn.astype(F), False)
        return s_up < lo, (s_dn > hi) & (d2f <= F(3e38))


def test_fp32_pretest_never_contradicts_the_fp64_test():
    rng = np.random.default_rng(11)
    n_fast = n_all = 0
    for _ in range(120):
        scale = 10.0 ** rng.uniform(-6, 6)
        off = rng.uniform(-3, 3) * scale * 10.0 ** rng.uniform(0, 7)
        level = int(rng.integers(1, 33))
        region = scale / 2.0 ** level
        theta = float(rng.choice([0.3, 0.5, 0.7, 1.0]))
        n = 16_384
        cx = off + rng.uniform(0, scale, n)
        cy = off + rng.uniform(0, scale, n)
        r = region / theta * (1 + rng.normal(0, 1, n) * 10.0 ** rng.uniform(-12, -1, n))
        ang = rng.uniform(0, 2 * np.pi, n)
        x = cx + r * np.cos(ang)
        y = cy + r * np.sin(ang)
        dx = x - cx
        dy = y - cy
        d2 = dx * dx + dy * dy
        mbx = np.full(n, region * region / (theta * theta * (1.0 + 2e-13)))
        mby = np.full(n, region * region / (theta * theta * (1.0 - 2e-13)))
        ref_open = np.where(d2 < mbx, True, np.where(d2 > mby, False, region > theta * np.sqrt(d2)))
        s_open, s_acc = _pretest(x, y, cx, cy, mbx, mby)
        assert not (s_open & ~ref_open).any()
        assert not (s_acc & ref_open).any()
        n_fast += int(s_open.sum() + s_acc.sum())
        n_all += n
    # the pairs sit near the boundary on purpose, yet most are decided in FP32
    assert n_fast > 0.2 * n_all
