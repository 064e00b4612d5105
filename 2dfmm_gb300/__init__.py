"""Host-side Python view of libtree2d_gb300.so (the GB300 vortex-blob treecode).

The product is the shared library with the C ABI declared in
include/tree2d.h; this module binds it with ctypes and mirrors the
reference's interface:

    make_tree(vor_b, cir_b, cor_b)     ver-c/src/quadtree.c:102-171
    biot_tree(x, y) -> (u, v)          ver-c/src/fmm.c:69-118

plus the library's extensions (parameters, modes, batch evaluation,
device-resident solves, tree export, statistics).  There is no fallback:
if the library is missing or has no GPU, calls raise.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libtree2d_gb300.so")

OK = 0
ERR_PARAM_FILE, ERR_BAD_PARAMS, ERR_BAD_INPUT, ERR_TOO_DEEP, ERR_CUDA, ERR_NO_TREE, ERR_NO_DEVICE, ERR_TIMEOUT, \
    ERR_MODE, ERR_TOO_LARGE, ERR_FILE = range(1, 12)
STATIC_MAX_BLOBS = 65536
MODE_PLAIN, MODE_MIXED, MODE_LEARNED = 0, 1, 2
EVAL_VARIANTS = 5  # TREE2D_EVAL_VARIANTS

# Every symbol include/tree2d.h declares.
EXPORTS = [
    "make_tree", "biot_tree", "tree2d_last_error", "tree2d_error_string", "tree2d_set_params",
    "tree2d_clear_params", "tree2d_get_params", "tree2d_set_mode", "tree2d_get_mode", "tree2d_set_mixed_params", "tree2d_set_mixed_leaf", "biot_tree_batch",
    "tree2d_solve_device", "tree2d_solve_device_static", "tree2d_solve_sets", "tree2d_set_tuning", "tree2d_set_level_chain", "tree2d_set_m2l_rows", "tree2d_get_stats", "tree2d_export_tree", "tree2d_direct_device", "tree2d_fp64_probe", "tree2d_pipe_probe", "tree2d_wait_probe", "tree2d_version",
    "tree2d_learn_param_count", "tree2d_learn_load", "tree2d_learn_set_weights", "tree2d_learn_set_envelope", "tree2d_learn_get_weights", "tree2d_learn_set_options", "tree2d_learn_set_far_orders",
    "tree2d_learn_collect", "tree2d_learn_train", "tree2d_mlp_grad", "tree2d_mlp_forward",
    "tree2d_set_mirror", "tree2d_advect_device",
]


class Tree2DError(RuntimeError):
    def __init__(self, code: int, where: str = ""):
        self.code = code
        super().__init__(f"{where}: tree2d error {code}: {error_string(code)}")


class Stats(ctypes.Structure):
    _fields_ = [
        ("n_blobs", ctypes.c_longlong), ("n_cells", ctypes.c_longlong), ("n_leaves", ctypes.c_longlong),
        ("depth", ctypes.c_int), ("mode", ctypes.c_int), ("n_m2s", ctypes.c_longlong),
        ("n_pairs", ctypes.c_longlong), ("n_m2l", ctypes.c_longlong), ("ms_build", ctypes.c_double),
        ("ms_upward", ctypes.c_double), ("ms_eval", ctypes.c_double), ("ms_total", ctypes.c_double),
        ("n_launches", ctypes.c_longlong), ("m2l_path", ctypes.c_int), ("eval_variant", ctypes.c_int),
        ("learned_active", ctypes.c_int), ("n_list_u", ctypes.c_longlong), ("n_list_k", ctypes.c_longlong),
        ("leaf_blobs", ctypes.c_int), ("n_list_k_blobs", ctypes.c_longlong),
        ("n_pairs_k", ctypes.c_longlong), ("n_pairs_k_listed", ctypes.c_longlong), ("m2l_rows", ctypes.c_int),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_lib = None


def build(verbose: bool = False) -> str:
    """Compiles the CUDA sources for sm_103a (see build.py)."""
    from importlib import import_module
    return import_module(__name__ + ".build").build(verbose=verbose)


def load(path: str | None = None):
    """Loads the library (raises if it is missing: there is no CPU fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it first (python -c 'import __graft_entry__ as g; g.build()')")
    L = ctypes.CDLL(path)
    L.make_tree.argtypes = [ctypes.c_int, _dp, _dp, _dp]
    L.make_tree.restype = None
    L.biot_tree.argtypes = [ctypes.c_double, ctypes.c_double, _dp, _dp]
    L.biot_tree.restype = None
    L.tree2d_last_error.restype = ctypes.c_int
    L.tree2d_error_string.argtypes = [ctypes.c_int]
    L.tree2d_error_string.restype = ctypes.c_char_p
    L.tree2d_set_params.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double]
    L.tree2d_set_params.restype = ctypes.c_int
    L.tree2d_clear_params.restype = None
    L.tree2d_get_params.argtypes = [_ip, _ip, _dp, _dp]
    L.tree2d_set_mode.argtypes = [ctypes.c_int]
    L.tree2d_set_mode.restype = ctypes.c_int
    L.tree2d_get_mode.restype = ctypes.c_int
    L.tree2d_set_mixed_params.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_int]
    L.tree2d_set_mixed_params.restype = ctypes.c_int
    L.tree2d_set_mixed_leaf.argtypes = [ctypes.c_int]
    L.tree2d_set_mixed_leaf.restype = ctypes.c_int
    L.biot_tree_batch.argtypes = [ctypes.c_int, _dp, _dp]
    L.biot_tree_batch.restype = ctypes.c_int
    L.tree2d_solve_device.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_void_p, ctypes.c_void_p]
    L.tree2d_solve_device.restype = ctypes.c_int
    L.tree2d_solve_device_static.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                             ctypes.c_void_p, ctypes.c_void_p]
    L.tree2d_solve_device_static.restype = ctypes.c_int
    L.tree2d_get_stats.argtypes = [ctypes.POINTER(Stats)]
    L.tree2d_get_stats.restype = ctypes.c_int
    L.tree2d_export_tree.argtypes = [_ip, ctypes.c_longlong, _ip, _ip, _ip, _ip, _dp, _dp, _dp, _dp]
    L.tree2d_export_tree.restype = ctypes.c_longlong
    L.tree2d_direct_device.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                       ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    L.tree2d_direct_device.restype = ctypes.c_int
    L.tree2d_fp64_probe.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, _dp]
    L.tree2d_fp64_probe.restype = ctypes.c_int
    L.tree2d_pipe_probe.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, _dp]
    L.tree2d_pipe_probe.restype = ctypes.c_int
    L.tree2d_set_tuning.argtypes = [ctypes.c_int, ctypes.c_int]
    L.tree2d_set_tuning.restype = ctypes.c_int
    L.tree2d_set_level_chain.argtypes = [ctypes.c_int]
    L.tree2d_set_level_chain.restype = ctypes.c_int
    L.tree2d_set_m2l_rows.argtypes = [ctypes.c_int]
    L.tree2d_set_m2l_rows.restype = ctypes.c_int
    L.tree2d_solve_sets.argtypes = [ctypes.c_int, _ip, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                    ctypes.c_void_p, ctypes.c_void_p]
    L.tree2d_solve_sets.restype = ctypes.c_int
    L.tree2d_wait_probe.argtypes = [ctypes.c_longlong, _ip]
    L.tree2d_wait_probe.restype = ctypes.c_int
    L.tree2d_version.restype = ctypes.c_char_p
    fp = ctypes.POINTER(ctypes.c_float)
    L.tree2d_learn_param_count.restype = ctypes.c_int
    L.tree2d_learn_load.argtypes = [ctypes.c_char_p]
    L.tree2d_learn_load.restype = ctypes.c_int
    L.tree2d_learn_set_weights.argtypes = [fp, ctypes.c_int]
    L.tree2d_learn_get_weights.argtypes = [fp, ctypes.c_int]
    L.tree2d_learn_set_options.argtypes = [ctypes.c_float, ctypes.c_int, ctypes.c_double]
    L.tree2d_learn_set_envelope.argtypes = [ctypes.c_double, ctypes.c_double]
    L.tree2d_learn_set_envelope.restype = ctypes.c_int
    L.tree2d_learn_collect.argtypes = [ctypes.c_int, ctypes.c_uint, fp, _ip]
    L.tree2d_learn_train.argtypes = [ctypes.c_int, fp, _ip, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                     ctypes.c_uint, fp]
    L.tree2d_mlp_grad.argtypes = [ctypes.c_int, fp, _ip, fp, fp, fp]
    L.tree2d_mlp_forward.argtypes = [ctypes.c_int, fp, fp, fp, ctypes.c_int]
    L.tree2d_set_mirror.argtypes = [ctypes.c_int, ctypes.c_double]
    L.tree2d_set_mirror.restype = ctypes.c_int
    L.tree2d_advect_device.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double,
                                       ctypes.c_void_p]
    L.tree2d_advect_device.restype = ctypes.c_int
    L.tree2d_learn_set_far_orders.argtypes = [ctypes.c_int]
    for f in ("tree2d_learn_set_weights", "tree2d_learn_get_weights", "tree2d_learn_set_options",
              "tree2d_learn_set_far_orders", "tree2d_learn_collect", "tree2d_learn_train", "tree2d_mlp_grad", "tree2d_mlp_forward"):
        getattr(L, f).restype = ctypes.c_int
    _lib = L
    return L


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _ptr(a):
    return a.ctypes.data_as(_dp)


def error_string(code: int) -> str:
    return load().tree2d_error_string(code).decode()


def last_error() -> int:
    return load().tree2d_last_error()


def _check(rc: int, where: str):
    if rc != OK:
        raise Tree2DError(rc, where)


def set_params(nterms: int, num_p: int, theta: float, r_min: float = 0.01):
    _check(load().tree2d_set_params(nterms, num_p, theta, r_min), "set_params")


def clear_params():
    load().tree2d_clear_params()


def get_params():
    a, b = ctypes.c_int(), ctypes.c_int()
    c, d = ctypes.c_double(), ctypes.c_double()
    load().tree2d_get_params(ctypes.byref(a), ctypes.byref(b), ctypes.byref(c), ctypes.byref(d))
    return a.value, b.value, c.value, d.value


def set_mode(mode: int):
    _check(load().tree2d_set_mode(mode), "set_mode")


def set_mixed_params(pterms: int = 16, cutoff_sigmas: float = 2.5, use_tensor_cores: bool = True):
    _check(load().tree2d_set_mixed_params(pterms, cutoff_sigmas, int(use_tensor_cores)), "set_mixed_params")


def set_mixed_leaf(max_blobs: int = -1):
    """Most blobs per leaf of the mixed forms' tree: -1 by set size (64 /
    96 / 128 from 512K / 2M blobs), 0 the parameters' num_p - 1, > 0 fixed."""
    _check(load().tree2d_set_mixed_leaf(max_blobs), "set_mixed_leaf")


def get_mode() -> int:
    return load().tree2d_get_mode()


def make_tree(vor_b, cir_b, cor_b, check: bool = True) -> int:
    """make_tree(nvor_b, vor_b, cir_b, cor_b) of the reference; vor_b is
    (n, 2) x,y per blob.  Returns the library status (the C call itself
    returns void, like the reference)."""
    xy = _f64(vor_b).reshape(-1, 2)
    cir = _f64(cir_b)
    cor = _f64(cor_b)
    n = len(cir)
    if xy.shape[0] != n or cor.shape[0] != n:
        raise ValueError("vor_b, cir_b and cor_b must describe the same number of blobs")
    L = load()
    L.make_tree(n, _ptr(xy), _ptr(cir), _ptr(cor))
    rc = L.tree2d_last_error()
    if check:
        _check(rc, "make_tree")
    return rc


def biot_tree(x: float, y: float):
    """Velocity (u, v) at one point, as the reference's biot_tree."""
    u, v = ctypes.c_double(), ctypes.c_double()
    load().biot_tree(float(x), float(y), ctypes.byref(u), ctypes.byref(v))
    return u.value, v.value


def biot_tree_batch(xy, check: bool = True, out=None):
    """Velocities at the points xy ((m, 2)); `out`, if given, is a C-contiguous
    float64 (m, 2) array that receives them (e.g. a page-locked buffer)."""
    xy = _f64(xy).reshape(-1, 2)
    if out is None:
        uv = np.empty_like(xy)
    else:
        uv = out
        if uv.dtype != np.float64 or uv.shape != xy.shape or not uv.flags.c_contiguous:
            raise ValueError("out must be a C-contiguous float64 array shaped like xy")
    rc = load().biot_tree_batch(len(xy), _ptr(xy), _ptr(uv))
    if check:
        _check(rc, "biot_tree_batch")
    return uv


def solve_device(d_xy: int, d_cir: int, d_cor: int, d_uv: int, n: int, stream: int = 0):
    """Device-resident solve over raw device pointers (ints)."""
    _check(load().tree2d_solve_device(n, d_xy, d_cir, d_cor, d_uv, stream or None), "solve_device")


def set_tuning(autotune: bool = True, eval_variant: int = -1):
    """Near-field kernel tuning (bit-identical variants): autotune on the
    first solve of each size class, or force a variant 0..EVAL_VARIANTS-1."""
    _check(load().tree2d_set_tuning(int(autotune), eval_variant), "set_tuning")


def set_level_chain(on: bool = False):
    """P = 16 M2M / L2L levels as one cooperative launch each, or one launch
    per level (default); the results are the same."""
    _check(load().tree2d_set_level_chain(int(on)), "set_level_chain")


def set_m2l_rows(rows: int = 0):
    """Cells per CTA of the tensor-core M2L: 128, 64 (bit-identical
    results), or 0 for the tuner's choice."""
    _check(load().tree2d_set_m2l_rows(int(rows)), "set_m2l_rows")


def solve_sets(d_xy: int, d_cir: int, d_cor: int, d_uv: int, offsets, stream: int = 0):
    """Batched mixed solve of independent sets in one tree (device pointers;
    `offsets` = nsets + 1 blob offsets, host)."""
    off = np.ascontiguousarray(offsets, dtype=np.int32)
    _check(load().tree2d_solve_sets(len(off) - 1, off.ctypes.data_as(_ip), d_xy, d_cir, d_cor, d_uv,
                                    stream or None), "solve_sets")


def solve_device_static(d_xy: int, d_cir: int, d_cor: int, d_uv: int, n: int, stream: int = 0) -> int:
    """The no-allocation variant of solve_device (scratch in a fixed device
    array; n <= STATIC_MAX_BLOBS).  Returns the status."""
    return load().tree2d_solve_device_static(n, d_xy, d_cir, d_cor, d_uv, stream or None)


def direct_device(d_txy: int, ntgt: int, d_sxy: int, d_cir: int, d_cor: int, nsrc: int, d_uv: int, stream: int = 0):
    _check(load().tree2d_direct_device(ntgt, d_txy, nsrc, d_sxy, d_cir, d_cor, d_uv, stream or None), "direct")


def stats() -> dict:
    s = Stats()
    _check(load().tree2d_get_stats(ctypes.byref(s)), "stats")
    return s.as_dict()


def export_tree(n: int, nterms: int) -> dict:
    """Permutation and non-empty cells below the root (pre-order) of the
    last make_tree, in the oracle's dump format."""
    L = load()
    nc = L.tree2d_export_tree(None, 0, None, None, None, None, None, None, None, None)
    if nc < 0:
        raise Tree2DError(ERR_NO_TREE, "export_tree")
    perm = np.empty(n, np.int32)
    lev, beg, end, leaf = (np.empty(nc, np.int32) for _ in range(4))
    cx, cy, reg = (np.empty(nc) for _ in range(3))
    coef = np.empty((nc, max(nterms, 1), 2))
    ip = lambda a: a.ctypes.data_as(_ip)  # noqa: E731
    got = L.tree2d_export_tree(ip(perm), max(nc, 1), ip(lev), ip(beg), ip(end), ip(leaf), _ptr(cx), _ptr(cy),
                               _ptr(reg), _ptr(coef))
    if got != nc:
        raise Tree2DError(ERR_CUDA, "export_tree")
    return dict(perm=perm, level=lev, begin=beg, end=end, leaf=leaf, cx=cx, cy=cy, region=reg,
                coef=(coef[..., 0] + 1j * coef[..., 1])[:, :nterms])


def fp64_peak_tflops(blocks: int = 152 * 8, iters: int = 20000, stream: int = 0) -> float:
    """Measured FP64 FMA throughput of this GPU (TFLOP/s, FMA = 2 flops)."""
    ms = ctypes.c_double()
    _check(load().tree2d_fp64_probe(blocks, iters, stream or None, ctypes.byref(ms)), "fp64_probe")
    return blocks * 256.0 * iters * 16.0 / (ms.value * 1e-3) / 1e12


def fp32_peak_tflops(blocks: int = 152 * 8, iters: int = 200000, stream: int = 0) -> float:
    """Measured FP32 FMA throughput of this GPU (TFLOP/s, FMA = 2 flops)."""
    ms = ctypes.c_double()
    _check(load().tree2d_pipe_probe(32, blocks, iters, stream or None, ctypes.byref(ms)), "pipe_probe")
    return blocks * 256.0 * iters * 16.0 / (ms.value * 1e-3) / 1e12


def wait_probe(polls: int = 100_000) -> int:
    """Runs the bounded-wait check kernel (a wait on a barrier nothing
    completes) and returns the status it recorded: TREE2D_ERR_TIMEOUT."""
    st = ctypes.c_int(-1)
    _check(load().tree2d_wait_probe(polls, ctypes.byref(st)), "wait_probe")
    return st.value


def set_mirror(enable: bool, d_mirror: float = 0.0):
    """Mirror wall at y = d_mirror (images as point vortices of opposite sign)."""
    _check(load().tree2d_set_mirror(int(enable), d_mirror), "set_mirror")


def advect_device(d_xy: int, d_uv: int, n: int, dt: float, stream: int = 0):
    """Forward Euler on device arrays: xy += dt * uv."""
    _check(load().tree2d_advect_device(n, d_xy, d_uv, dt, stream or None), "advect_device")


# ---------------------------------------------------------------- learned form

def _fp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def learn_param_count() -> int:
    return load().tree2d_learn_param_count()


def learn_load(path: str) -> int:
    """Loads a .t2dw weights file (parameters and training envelope) through
    the C loader; returns the status."""
    return load().tree2d_learn_load(os.fsencode(path))


def learn_set_weights(theta):
    th = np.ascontiguousarray(theta, np.float32)
    _check(load().tree2d_learn_set_weights(_fp(th), len(th)), "learn_set_weights")


def learn_get_weights():
    th = np.empty(learn_param_count(), np.float32)
    _check(load().tree2d_learn_get_weights(_fp(th), len(th)), "learn_get_weights")
    return th


def learn_set_options(direct_bias: float = 1.0, order_margin: int = 1, budget: float = 3e-7):
    _check(load().tree2d_learn_set_options(direct_bias, order_margin, budget), "learn_set_options")


def learn_set_far_orders(on: bool = False):
    """Learned form: the network also sets each W-list M2P's order (leaf
    sources), or (off) they all keep the full order."""
    _check(load().tree2d_learn_set_far_orders(int(on)), "learn_set_far_orders")


def learn_set_envelope(k_blobs_per_leaf_max: float, cutoff_sigmas: float = 0.0):
    """Training envelope: the largest mean number of source blobs in a
    leaf's K-list leaves that the network was trained on, counted at
    correction radius `cutoff_sigmas` (0: the radius in force); denser
    solves run the fixed mixed form."""
    _check(load().tree2d_learn_set_envelope(k_blobs_per_leaf_max, cutoff_sigmas), "learn_set_envelope")


def learn_collect(max_samples: int, seed: int = 0):
    X = np.empty((max_samples, 16), np.float32)
    y = np.empty(max_samples, np.int32)
    n = load().tree2d_learn_collect(max_samples, seed, _fp(X), y.ctypes.data_as(_ip))
    if n < 0:
        raise Tree2DError(-n, "learn_collect")
    return X[:n].copy(), y[:n].copy()


def learn_train(X, y, steps: int = 1000, batch: int = 4096, lr: float = 2e-3, seed: int = 0) -> float:
    X = np.ascontiguousarray(X, np.float32)
    y = np.ascontiguousarray(y, np.int32)
    loss = np.zeros(1, np.float32)
    _check(load().tree2d_learn_train(len(y), _fp(X), y.ctypes.data_as(_ip), steps, batch, lr, seed, _fp(loss)),
           "learn_train")
    return float(loss[0])


def mlp_grad(X, y, theta):
    X = np.ascontiguousarray(X, np.float32)
    y = np.ascontiguousarray(y, np.int32)
    th = np.ascontiguousarray(theta, np.float32)
    g = np.empty_like(th)
    loss = np.zeros(1, np.float32)
    _check(load().tree2d_mlp_grad(len(y), _fp(X), y.ctypes.data_as(_ip), _fp(th), _fp(g), _fp(loss)), "mlp_grad")
    return float(loss[0]), g


def mlp_forward(X, theta, tensor_cores: bool = False):
    X = np.ascontiguousarray(X, np.float32)
    th = np.ascontiguousarray(theta, np.float32)
    out = np.empty((len(X), 16), np.float32)
    _check(load().tree2d_mlp_forward(len(X), _fp(X), _fp(th), _fp(out), int(tensor_cores)), "mlp_forward")
    return out


def version() -> str:
    return load().tree2d_version().decode()
