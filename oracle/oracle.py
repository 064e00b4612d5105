"""ctypes view of the CPU oracle (``liboracle.so``, built from tree2d_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, by ``__graft_entry__.smoke``
(as the checker) and by ``bench.py`` (as the timed CPU baseline).  The
product library never imports this module.

The oracle restates the reference treecode (ver-c/src/quadtree.c,
ver-c/src/fmm.c, ver-c/src/morton_order.c); see the header of
tree2d_oracle.c for the file:line map.  It is pinned bit-exact against the
reference built from its own sources (golden vectors in tests/golden/).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_DRIVER = os.path.join(HERE, "_ref", "ref_driver")

_lock = threading.Lock()
_lib = None

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_lp = ctypes.POINTER(ctypes.c_long)


def build(force: bool = False) -> str:
    """Compiles liboracle.so with the recipe in oracle/Makefile."""
    srcs = [os.path.join(HERE, f) for f in ("tree2d_oracle.c", "tree2d_sparse.c")]
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < max(map(os.path.getmtime, srcs)):
        subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    return LIB_PATH


REF_STAGE = os.path.join(HERE, "_ref", "src")
REF_FILES = ("quadtree.c", "quadtree.h", "fmm.c", "fmm.h", "morton_order.c", "morton_order.h")


def reference_sources(ref_src: str | None = None) -> str | None:
    """Directory holding the reference's ver-c/src files: `ref_src` or
    $TREE2D_REF_SRC when given and present, else the unmodified copy staged
    in _ref/src (git-ignored; it travels with the working tree to a machine
    without the reference), else None."""
    for cand in (ref_src, os.environ.get("TREE2D_REF_SRC")):
        if cand and all(os.path.isfile(os.path.join(cand, f)) for f in REF_FILES):
            return cand
    if all(os.path.isfile(os.path.join(REF_STAGE, f)) for f in REF_FILES):
        return REF_STAGE
    return None


def build_reference(ref_src: str | None = None) -> str | None:
    """Builds _ref/ref_driver from the reference's own sources when they are
    available (see reference_sources); a given source directory is first
    staged, unmodified, into _ref/src so that the build can be repeated where
    the reference is absent.  Returns the driver's path or None."""
    src = reference_sources(ref_src)
    if src is None:
        return None
    if os.path.abspath(src) != os.path.abspath(REF_STAGE):
        subprocess.run(["make", "-s", "-C", HERE, "stage", f"REF_SRC={src}"], check=True)
    subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)
    if not _runs(REF_DRIVER):  # built for another machine: rebuild here
        subprocess.run(["make", "-s", "-B", "-C", HERE, "ref"], check=True)
    return REF_DRIVER


def _runs(path: str) -> bool:
    try:
        return subprocess.run([path], capture_output=True).returncode == 2  # its usage exit
    except OSError:
        return False


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(LIB_PATH)
            L.ora_set_params.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double]
            L.ora_make_tree.argtypes = [ctypes.c_int, _dp, _dp, _dp, ctypes.c_char_p, ctypes.c_int]
            L.ora_make_tree.restype = ctypes.c_int
            L.ora_biot_tree.argtypes = [ctypes.c_double, ctypes.c_double, _dp, _dp]
            L.ora_biot_many.argtypes = [ctypes.c_int, _dp, _dp, ctypes.c_int, _lp, _lp]
            L.ora_levels.restype = ctypes.c_int
            L.ora_num_nodes.restype = ctypes.c_long
            L.ora_dump_tree.argtypes = [_ip, ctypes.c_long, _ip, _ip, _ip, _ip, _dp, _dp, _dp, _dp]
            L.ora_dump_tree.restype = ctypes.c_long
            L.ora_direct.argtypes = [ctypes.c_int, _dp, ctypes.c_int, _dp, _dp, _dp, _dp, ctypes.c_int]
            L.ora_max_threads.restype = ctypes.c_int
            L.ora_sp_make_tree.argtypes = [ctypes.c_int, _dp, _dp, _dp, ctypes.c_int]
            L.ora_sp_make_tree.restype = ctypes.c_int
            L.ora_sp_levels.restype = ctypes.c_int
            L.ora_sp_num_nodes.restype = ctypes.c_long
            L.ora_sp_biot_many.argtypes = [ctypes.c_int, _dp, _dp, ctypes.c_int, _lp, _lp]
            L.ora_sp_biot_ext.argtypes = [ctypes.c_int, _dp, _dp, _dp, ctypes.c_int]
            L.ora_sp_dump_tree.argtypes = [_ip, ctypes.c_long, _ip, _ip, _ip, _ip, _dp, _dp, _dp, _dp]
            L.ora_sp_dump_tree.restype = ctypes.c_long
            _lib = L
    return _lib


def _p(a, t=_dp):
    return a.ctypes.data_as(t)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class Oracle:
    """One oracle tree (the oracle keeps process-global state, like the
    reference; only one tree exists at a time)."""

    def __init__(self, nterms: int, num_p: int, theta: float, r_min: float = 0.01, fresh: bool = True):
        self.L = lib()
        self.L.ora_set_params(nterms, num_p, theta, r_min)
        if fresh:
            self.L.ora_reset()
        self.nterms = nterms

    def make_tree(self, xy, cir, cor, max_level_cap: int = 24) -> int:
        xy = _f64(xy).reshape(-1, 2)
        cir = _f64(cir)
        cor = _f64(cor)
        self._keep = (xy, cir, cor)
        rc = self.L.ora_make_tree(len(cir), _p(xy), _p(cir), _p(cor), None, max_level_cap)
        if rc != 0:
            raise RuntimeError(f"oracle make_tree failed: {rc}")
        return rc

    def biot(self, txy, threads: int = 0, counters: bool = False):
        txy = _f64(txy).reshape(-1, 2)
        uv = np.empty_like(txy)
        a = ctypes.c_long(0)
        b = ctypes.c_long(0)
        self.L.ora_biot_many(len(txy), _p(txy), _p(uv), threads, ctypes.byref(a), ctypes.byref(b))
        if counters:
            return uv, a.value, b.value
        return uv

    def levels(self) -> int:
        return self.L.ora_levels()

    def close(self):
        """Releases the tree (tens of GB for deep dense trees)."""
        self.L.ora_free()

    def num_nodes(self) -> int:
        return self.L.ora_num_nodes()

    def dump(self, n: int):
        """Permutation and non-empty cells (pre-order, root excluded)."""
        nc = self.L.ora_dump_tree(None, 0, None, None, None, None, None, None, None, None)
        perm = np.empty(n, np.int32)
        lev = np.empty(nc, np.int32)
        beg = np.empty(nc, np.int32)
        end = np.empty(nc, np.int32)
        leaf = np.empty(nc, np.int32)
        cx = np.empty(nc)
        cy = np.empty(nc)
        reg = np.empty(nc)
        coef = np.empty((nc, self.nterms, 2))
        self.L.ora_dump_tree(_p(perm, _ip), nc, _p(lev, _ip), _p(beg, _ip), _p(end, _ip), _p(leaf, _ip),
                             _p(cx), _p(cy), _p(reg), _p(coef))
        return dict(perm=perm, level=lev, begin=beg, end=end, leaf=leaf, cx=cx, cy=cy, region=reg,
                    coef=coef[..., 0] + 1j * coef[..., 1])


class SparseOracle:
    """The reference tree built without the dense node array
    (tree2d_sparse.c): the same tree, coefficients and velocities as Oracle,
    for trees too deep for the dense layout, plus the treecode's value in
    extended precision.  One sparse tree exists at a time."""

    def __init__(self, nterms: int, num_p: int, theta: float, r_min: float = 0.01):
        self.L = lib()
        self.L.ora_set_params(nterms, num_p, theta, r_min)
        self.nterms = nterms

    def make_tree(self, xy, cir, cor, level_cap: int = 60) -> int:
        xy = _f64(xy).reshape(-1, 2)
        cir = _f64(cir)
        cor = _f64(cor)
        rc = self.L.ora_sp_make_tree(len(cir), _p(xy), _p(cir), _p(cor), level_cap)
        if rc != 0:
            raise RuntimeError(f"sparse oracle make_tree failed: {rc}")
        return rc

    def levels(self) -> int:
        return self.L.ora_sp_levels()

    def biot(self, txy, threads: int = 0, counters: bool = False):
        txy = _f64(txy).reshape(-1, 2)
        uv = np.empty_like(txy)
        a = ctypes.c_long(0)
        b = ctypes.c_long(0)
        self.L.ora_sp_biot_many(len(txy), _p(txy), _p(uv), threads, ctypes.byref(a), ctypes.byref(b))
        return (uv, a.value, b.value) if counters else uv

    def biot_ext(self, txy, threads: int = 0, cond: bool = False):
        """The same treecode (same accepted cells and pairs) evaluated in
        extended precision: its value to far below FP64 rounding.  With
        cond=True also the sum of its contributions' magnitudes per target
        (the scale of any FP64 evaluation's rounding error)."""
        txy = _f64(txy).reshape(-1, 2)
        uv = np.empty_like(txy)
        c = np.empty(len(txy))
        self.L.ora_sp_biot_ext(len(txy), _p(txy), _p(uv), _p(c), threads)
        return (uv, c) if cond else uv

    def dump(self, n: int):
        nc = self.L.ora_sp_dump_tree(None, 0, None, None, None, None, None, None, None, None)
        perm = np.empty(n, np.int32)
        lev, beg, end, leaf = (np.empty(nc, np.int32) for _ in range(4))
        cx, cy, reg = (np.empty(nc) for _ in range(3))
        coef = np.empty((nc, self.nterms, 2))
        self.L.ora_sp_dump_tree(_p(perm, _ip), nc, _p(lev, _ip), _p(beg, _ip), _p(end, _ip), _p(leaf, _ip),
                                _p(cx), _p(cy), _p(reg), _p(coef))
        return dict(perm=perm, level=lev, begin=beg, end=end, leaf=leaf, cx=cx, cy=cy, region=reg,
                    coef=coef[..., 0] + 1j * coef[..., 1])

    def close(self):
        self.L.ora_sp_reset()


def direct(txy, sxy, cir, cor, threads: int = 0):
    """FP64 direct sum of the regularised Biot-Savart kernel (the accuracy yardstick)."""
    L = lib()
    txy = _f64(txy).reshape(-1, 2)
    sxy = _f64(sxy).reshape(-1, 2)
    cir = _f64(cir)
    cor = _f64(cor)
    uv = np.empty_like(txy)
    L.ora_direct(len(txy), _p(txy), len(cir), _p(sxy), _p(cir), _p(cor), _p(uv), threads)
    return uv


def max_threads() -> int:
    return lib().ora_max_threads()


# ---------------------------------------------------------------------------
# reference driver (only where the reference sources were available to build it)

def write_input(path, xy, cir, cor, txy):
    xy = _f64(xy).reshape(-1, 2)
    txy = _f64(txy).reshape(-1, 2)
    with open(path, "wb") as f:
        np.array([len(cir), len(txy)], np.int32).tofile(f)
        xy.tofile(f)
        _f64(cir).tofile(f)
        _f64(cor).tofile(f)
        txy.tofile(f)


def read_output(path):
    with open(path, "rb") as f:
        n, nt, nc, nterms, max_level = np.fromfile(f, np.int32, 5)
        uv = np.fromfile(f, np.float64, 2 * nt).reshape(nt, 2)
        perm = np.fromfile(f, np.int32, n)
        lev, beg, end, leaf = (np.fromfile(f, np.int32, nc) for _ in range(4))
        cx, cy, reg = (np.fromfile(f, np.float64, nc) for _ in range(3))
        coef = np.fromfile(f, np.float64, nc * nterms * 2).reshape(nc, nterms, 2)
    return dict(uv=uv, perm=perm, level=lev, begin=beg, end=end, leaf=leaf, cx=cx, cy=cy, region=reg,
                coef=coef[..., 0] + 1j * coef[..., 1], max_level=int(max_level))


def reference_available() -> bool:
    """The reference's own build (_ref/ref_driver) exists and runs here."""
    return os.path.exists(REF_DRIVER) and _runs(REF_DRIVER)


def time_reference(workdir, xy, cir, cor, txy, nterms, num_p, theta, threads=1, batches=1):
    """Times the reference's own code on this machine: make_tree over all
    blobs once, then `batches` evaluations of the targets `txy` over
    `threads` OpenMP threads, in a fresh process.  Returns (make_tree
    seconds, [seconds per batch], max level)."""
    import re
    out = run_reference(workdir, xy, cir, cor, txy, nterms, num_p, theta, threads=threads, batches=batches)
    log = out["log"]
    m = re.search(r"make_tree ([0-9.]+) s", log)
    per = [float(x) for x in re.findall(r"batch \d+ biot_tree ([0-9.]+) s", log)]
    if not per:
        per = [float(re.search(r"biot_tree ([0-9.]+) s", log).group(1))]
    return float(m.group(1)), per, out["max_level"]


def run_reference(workdir, xy, cir, cor, txy, nterms, num_p, theta, r_min=0.01, threads=1, batches=1):
    """Runs the reference (built from its sources) in a fresh process.

    The reference reads ../cal_cond/fmm_param.dat relative to its working
    directory (ver-c/src/quadtree.c:12-27), so that file is written first."""
    if not os.path.exists(REF_DRIVER):
        raise FileNotFoundError(REF_DRIVER)
    run = os.path.join(workdir, "run")
    cc = os.path.join(workdir, "cal_cond")
    os.makedirs(run, exist_ok=True)
    os.makedirs(cc, exist_ok=True)
    with open(os.path.join(cc, "fmm_param.dat"), "w") as f:
        f.write(f"{nterms}    nterms\n{num_p}   num_p\n{theta!r} theta\n{r_min!r}  r_min ! for Tree\n")
    fin = os.path.join(workdir, "in.bin")
    fout = os.path.join(workdir, "out.bin")
    write_input(fin, xy, cir, cor, txy)
    env = dict(os.environ)
    p = subprocess.run(["bash", "-c", f"ulimit -s unlimited; exec {REF_DRIVER} {fin} {fout} {threads} {batches}"],
                       cwd=run, env=env, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"reference driver failed ({p.returncode}): {p.stderr}")
    out = read_output(fout)
    out["log"] = p.stderr.strip()
    return out
