"""Seeded synthetic blob sets for the benchmark configurations, and a reader
for the vortex solver's snapshot files.

All generators use numpy's PCG64 (``default_rng``), whose streams are the
same on every platform, so a (config, seed) pair names one exact input.

Parameter conventions follow the reference: ``nterms`` is the number of
stored coefficients (S2M/M2M fill nterms, M2S sums nterms-1 terms,
ver-c/src/fmm.c:24,48,64), so expansion order p means nterms = p+1; a leaf
holds fewer than ``num_p`` blobs (ver-c/src/quadtree.c:240), so "at most M
blobs per leaf" means num_p = M+1.
"""
from __future__ import annotations

import dataclasses
import struct

import numpy as np


@dataclasses.dataclass
class BlobSet:
    name: str
    xy: np.ndarray      # (n, 2) float64, x and y interleaved per blob
    cir: np.ndarray     # (n,) float64 circulation
    cor: np.ndarray     # (n,) float64 core radius
    nterms: int
    num_p: int
    theta: float
    stored_fp32: bool = False

    @property
    def n(self) -> int:
        return len(self.cir)


def uniform(n=20_000, seed=1, sigma=0.005, nterms=11, num_p=33, theta=0.5, name="uniform"):
    """Config 1 (20,000 blobs, U[0,1]^2, Gamma ~ N(0,1)/N, sigma 0.005, p=10,
    at most 32 blobs per leaf, theta 0.5) at any size."""
    rng = np.random.default_rng(seed)
    xy = rng.random((n, 2))
    cir = rng.standard_normal(n) / n
    cor = np.full(n, sigma)
    return BlobSet(name, xy, cir, cor, nterms, num_p, theta)


def lamb_oseen(n=1_048_576, seed=2, sigma=0.002, nterms=13, num_p=65, theta=0.5, name="lamb_oseen"):
    """Config 2: r ~ Rayleigh(0.1) about (0.5,0.5), angle U[0,2pi),
    Gamma ~ exp(-r^2/0.02) normalised to total 1, sigma 0.002, p=12,
    at most 64 blobs per leaf, theta 0.5."""
    rng = np.random.default_rng(seed)
    r = rng.rayleigh(0.1, n)
    a = rng.random(n) * 2.0 * np.pi
    xy = np.stack([0.5 + r * np.cos(a), 0.5 + r * np.sin(a)], axis=1)
    g = np.exp(-r * r / 0.02)
    cir = g / g.sum()
    cor = np.full(n, sigma)
    return BlobSet(name, xy, cir, cor, nterms, num_p, theta)


def two_patch_sheet(n=4_194_304, seed=3, sigma=0.001, nterms=13, num_p=65, theta=0.5, name="two_patch_sheet"):
    """Config 3: 45%/45% Gaussian patches (std 0.05) at (0.4,0.5) and
    (0.6,0.5) with Gamma = |N(0,1)|; 10% on the sheet
    y = 0.2 + 0.01 sin(8 pi x), x ~ U[0,1], Gamma = -1/N_sheet.  Positions
    and circulations are stored as FP32 (held here widened to FP64, exactly);
    sigma 0.001, p=12, theta 0.5.  The leaf size is not given by the
    configuration; 64 blobs (num_p 65) is used, as for config 2."""
    rng = np.random.default_rng(seed)
    n1 = int(round(0.45 * n))
    n2 = n1
    ns = n - n1 - n2
    p1 = rng.normal(0.0, 0.05, (n1, 2)) + np.array([0.4, 0.5])
    p2 = rng.normal(0.0, 0.05, (n2, 2)) + np.array([0.6, 0.5])
    sx = rng.random(ns)
    sy = 0.2 + 0.01 * np.sin(8.0 * np.pi * sx)
    xy = np.concatenate([p1, p2, np.stack([sx, sy], axis=1)])
    cir = np.concatenate([np.abs(rng.standard_normal(n1 + n2)), np.full(ns, -1.0 / ns)])
    xy = xy.astype(np.float32).astype(np.float64)
    cir = cir.astype(np.float32).astype(np.float64)
    cor = np.full(n, np.float64(np.float32(sigma)))
    return BlobSet(name, xy, cir, cor, nterms, num_p, theta, stored_fp32=True)


def batch_sets(nsets=512, seed=4, lo=2048, hi=200_000, nterms=11, num_p=33, theta=0.5):
    """Config 4: `nsets` independent sets, sizes log-uniform in [lo, hi],
    each uniform in its own [0,1]^2, Gamma ~ N(0,1)/N, sigma = 0.5/sqrt(N),
    p=10, theta 0.5 (leaf size 32, as config 1)."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(lo), np.log(hi), nsets)).astype(np.int64)
    sets = []
    for i, n in enumerate(sizes):
        n = int(n)
        xy = rng.random((n, 2))
        cir = rng.standard_normal(n) / n
        cor = np.full(n, 0.5 / np.sqrt(n))
        sets.append(BlobSet(f"set{i}", xy, cir, cor, nterms, num_p, theta))
    return sets


def sample_targets(n, k, seed=7):
    """k target indices drawn without replacement from n blobs (seeded)."""
    rng = np.random.default_rng(seed)
    k = min(k, n)
    return np.sort(rng.choice(n, size=k, replace=False))


def write_snapshot(path, xy, cir, cor, header_records=4):
    """Writes blobs in the snapshot's blob-block layout (Fortran unformatted
    sequential records: nvor_b, then per blob x,y | three velocity pairs |
    cir | cor | id), after `header_records` placeholder records standing for
    the solver's header (read_snapshot skips them by pattern)."""
    xy = np.asarray(xy, np.float64).reshape(-1, 2)
    cir = np.asarray(cir, np.float64)
    cor = np.asarray(cor, np.float64)

    def rec(f, payload):
        f.write(struct.pack("<i", len(payload)))
        f.write(payload)
        f.write(struct.pack("<i", len(payload)))

    with open(path, "wb") as f:
        for k in range(header_records):
            rec(f, struct.pack("<2d", float(k), 0.0))
        rec(f, struct.pack("<i", len(cir)))
        zero = struct.pack("<2d", 0.0, 0.0)
        for j in range(len(cir)):
            rec(f, struct.pack("<2d", xy[j, 0], xy[j, 1]))
            rec(f, zero)
            rec(f, zero)
            rec(f, zero)
            rec(f, struct.pack("<d", cir[j]))
            rec(f, struct.pack("<d", cor[j]))
            rec(f, struct.pack("<i", j + 1))


def read_snapshot(path):
    """Reads the blob block of a vortex-solver snapshot (``s_*****_step.dat``,
    Fortran unformatted sequential records, written by the solver's
    f_data_out.f90).  The blob block is the record holding nvor_b followed
    by nvor_b groups of 7 records (x,y | 3 velocity pairs | cir | cor | id);
    it is located by that record pattern.  Returns (xy, cir, cor)."""
    with open(path, "rb") as f:
        d = f.read()
    recs = []
    o = 0
    while o + 4 <= len(d):
        (ln,) = struct.unpack_from("<i", d, o)
        recs.append((o + 4, ln))
        o += 8 + ln
    lens = [ln for _, ln in recs]
    pat = [16, 16, 16, 16, 8, 8, 4]
    for i in range(len(lens) - 8):
        if lens[i] == 4 and lens[i + 1:i + 8] == pat:
            (nb,) = struct.unpack_from("<i", d, recs[i][0])
            if nb <= 0 or i + 1 + 7 * nb > len(recs):
                continue
            xy = np.empty((nb, 2))
            cir = np.empty(nb)
            cor = np.empty(nb)
            for j in range(nb):
                base = i + 1 + 7 * j
                xy[j] = struct.unpack_from("<2d", d, recs[base][0])
                (cir[j],) = struct.unpack_from("<d", d, recs[base + 4][0])
                (cor[j],) = struct.unpack_from("<d", d, recs[base + 5][0])
            return xy, cir, cor
    raise ValueError("no blob block found")
