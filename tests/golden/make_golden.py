"""Generates the golden vectors in this directory by running the REFERENCE
implementation, built from its own C sources (ver-c/src/quadtree.c,
fmm.c, morton_order.c) by oracle/Makefile's `ref` target, in a fresh
process per case.

Run here, where the reference sources are present:

    python tests/golden/make_golden.py [/path/to/reference]

Each case file <name>.npz holds the inputs (xy, cir, cor, targets), the
parameters, and what the reference computed: u,v at every target, the blob
permutation (leaves in depth-first quadrant order), and every non-empty cell
below the root in pre-order (level, [begin,end), leaf flag, centre, side,
coefficients after M2M).
"""
from __future__ import annotations

import importlib
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402

W = importlib.import_module("2dfmm_gb300.workloads")


def off_blob_targets(n, lo=-0.2, hi=1.2, seed=11):
    rng = np.random.default_rng(seed)
    return lo + (hi - lo) * rng.random((n, 2))


def cases(refdir):
    out = []
    # tiny and edge cases (cfg1 parameters)
    rng = np.random.default_rng(21)
    for n in (1, 2, 7, 32, 33):
        xy = rng.random((n, 2))
        out.append((f"tiny{n}", xy, rng.standard_normal(n) / max(n, 1), np.full(n, 0.005),
                    np.concatenate([xy, off_blob_targets(8, seed=n)]), 11, 33, 0.5))
    # coincident blobs (fewer than num_p at one point) and targets on blobs
    xy = rng.random((600, 2))
    xy[100:110] = xy[5]
    xy[200:203] = xy[7]
    out.append(("coincident", xy, rng.standard_normal(600) / 600, np.full(600, 0.005),
                np.concatenate([xy, off_blob_targets(16, seed=3)]), 11, 33, 0.5))
    # axis-aligned lattice: many blobs exactly on cell boundaries (>=, <= ties)
    g = np.arange(24) / 23.0
    xy = np.stack(np.meshgrid(g, g), -1).reshape(-1, 2)
    out.append(("lattice", xy, rng.standard_normal(len(xy)) / len(xy), np.full(len(xy), 0.01),
                np.concatenate([xy, off_blob_targets(16, seed=4)]), 9, 17, 0.5))
    # uniform 2000
    b = W.uniform(2000, seed=5)
    out.append(("u2k", b.xy, b.cir, b.cor, np.concatenate([b.xy, off_blob_targets(200)]), b.nterms, b.num_p,
                b.theta))
    # config 1, full size
    b = W.uniform()
    out.append(("cfg1", b.xy, b.cir, b.cor, np.concatenate([b.xy, off_blob_targets(200)]), b.nterms, b.num_p,
                b.theta))
    # config 2 distribution at 30,000 blobs (nterms 13, num_p 65)
    b = W.lamb_oseen(30_000, seed=6)
    out.append(("lamb30k", b.xy, b.cir, b.cor, b.xy, b.nterms, b.num_p, b.theta))
    # real solver snapshot, shipped parameters of ver-c/cal_cond/fmm_param.dat
    snap = os.path.join(refdir, "ver-c", "s_file", "s_00198_step.dat")
    if os.path.exists(snap):
        xy, cir, cor = W.read_snapshot(snap)
        out.append(("snapshot198", xy, cir, cor, xy, 15, 250, 0.5))
    return out


def main(refdir=None):
    """`refdir` (or $TREE2D_REF_ROOT) is the reference checkout, the directory
    that holds ver-c/."""
    refdir = refdir or os.environ.get("TREE2D_REF_ROOT")
    if not refdir:
        raise SystemExit("usage: make_golden.py <reference checkout>  (or set TREE2D_REF_ROOT)")
    drv = O.build_reference(os.path.join(refdir, "ver-c", "src"))
    if drv is None:
        raise SystemExit("reference sources not found")
    for name, xy, cir, cor, txy, nterms, num_p, theta in cases(refdir):
        with tempfile.TemporaryDirectory() as d:
            r = O.run_reference(d, xy, cir, cor, txy, nterms, num_p, theta, threads=os.cpu_count() or 1)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), xy=np.asarray(xy, np.float64),
                            cir=np.asarray(cir, np.float64), cor=np.asarray(cor, np.float64),
                            txy=np.asarray(txy, np.float64), nterms=nterms, num_p=num_p, theta=theta,
                            uv=r["uv"], perm=r["perm"], level=r["level"], begin=r["begin"], end=r["end"],
                            leaf=r["leaf"], cx=r["cx"], cy=r["cy"], region=r["region"], coef=r["coef"],
                            max_level=r["max_level"])
        print(name, len(cir), "targets", len(txy), "cells", len(r["level"]), r["log"])


if __name__ == "__main__":
    main(*sys.argv[1:])
