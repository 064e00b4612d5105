"""The C-ABI library without a GPU: it loads, exports every function
include/tree2d.h declares, and its host-side logic (parameters, errors,
parameter file) behaves as the reference's make_tree/biot_tree do."""
from __future__ import annotations

import ctypes
import os
import re

import numpy as np

from conftest import ROOT, pkg

HEADER = os.path.join(ROOT, "include", "tree2d.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"\b([A-Za-z_]\w*)\s*\([^;{]*\)\s*;", src)
    return sorted(set(n for n in names if n not in ("if", "while", "return")))


def test_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert {"make_tree", "biot_tree", "biot_tree_batch", "tree2d_solve_device"} <= set(names)
    for n in names:
        assert hasattr(lib, n), f"{n} not exported"
    assert set(names) == set(pkg().EXPORTS)


def test_version_and_errors(lib):
    P = pkg()
    assert "sm_103a" in P.version()
    for code in range(0, 12):
        assert P.error_string(code)


def test_param_validation(lib):
    P = pkg()
    assert lib.tree2d_set_params(1, 33, 0.5, 0.0) == 0
    assert lib.tree2d_set_params(40, 33, 0.5, 0.0) == P.ERR_BAD_PARAMS
    assert lib.tree2d_set_params(11, 1, 0.5, 0.0) == P.ERR_BAD_PARAMS
    assert lib.tree2d_set_params(11, 33, float("nan"), 0.0) == P.ERR_BAD_PARAMS
    assert lib.tree2d_set_params(11, 33, 0.5, 0.01) == 0
    assert P.get_params() == (11, 33, 0.5, 0.01)
    assert lib.tree2d_set_mode(7) == P.ERR_MODE
    assert lib.tree2d_set_mixed_leaf(-2) == P.ERR_BAD_PARAMS
    assert lib.tree2d_set_mixed_leaf(65536) == P.ERR_BAD_PARAMS
    assert lib.tree2d_set_mixed_leaf(100) == 0 and lib.tree2d_set_mixed_leaf(-1) == 0
    assert lib.tree2d_set_m2l_rows(32) == P.ERR_BAD_PARAMS and lib.tree2d_set_m2l_rows(-1) == P.ERR_BAD_PARAMS
    assert lib.tree2d_set_m2l_rows(64) == 0 and lib.tree2d_set_m2l_rows(128) == 0 and lib.tree2d_set_m2l_rows(0) == 0
    assert lib.tree2d_learn_set_envelope(-1.0, 3.0) == P.ERR_BAD_PARAMS
    assert lib.tree2d_learn_set_envelope(1.0, -3.0) == P.ERR_BAD_PARAMS
    assert lib.tree2d_learn_set_envelope(0.0, 0.0) == 0
    P.clear_params()


def test_biot_tree_without_tree_gives_nan(lib):
    P = pkg()
    lib.make_tree(-1, None, None, None)  # a failed make_tree leaves no tree (whatever ran before)
    assert P.last_error() != 0
    u, v = P.biot_tree(0.1, 0.2)
    assert np.isnan(u) and np.isnan(v)
    uv = P.biot_tree_batch(np.zeros((3, 2)), check=False)
    assert np.isnan(uv).all()


def test_param_file_read_like_reference(lib, tmp_path, monkeypatch):
    """make_tree reads ../cal_cond/fmm_param.dat relative to the working
    directory (quadtree.c:12-27), Fortran literal quirk included."""
    P = pkg()
    (tmp_path / "cal_cond").mkdir()
    (tmp_path / "run").mkdir()
    (tmp_path / "cal_cond" / "fmm_param.dat").write_text(
        "15    nterms\n250   num_p\n0.5d0 theta\n0.01  r_min ! for Tree\n")
    monkeypatch.chdir(tmp_path / "run")
    P.set_params(5, 9, 0.3, 0.0)
    P.clear_params()
    rc = P.make_tree(np.zeros((4, 2)), np.ones(4), np.ones(4), check=False)
    nterms, num_p, theta, _ = P.get_params()
    assert (nterms, num_p, theta) == (15, 250, 0.5)
    # without a GPU the call stops after reading the parameters
    assert rc in (P.OK, P.ERR_NO_DEVICE, P.ERR_CUDA)


def test_bad_input_rejected(lib):
    P = pkg()
    P.set_params(11, 33, 0.5)
    lib.make_tree(-1, None, None, None)
    assert P.last_error() == P.ERR_BAD_INPUT
    P.clear_params()


def test_c_caller_compiles_and_links(lib, tmp_path):
    """A C99 program (the reference's own language) includes the header with
    strict warnings, links the library and gets the reference's behaviour for
    biot_tree before any make_tree (NaN, with a status), without a GPU."""
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        import pytest
        pytest.skip("no C compiler")
    src = tmp_path / "main.c"
    src.write_text(
        "#include <stdio.h>\n"
        "#include \"tree2d.h\"\n"
        "int main(void) {\n"
        "  double u = 0.0, v = 0.0;\n"
        "  biot_tree(0.5, 0.5, &u, &v);\n"
        "  printf(\"%d %d %d\\n\", tree2d_last_error(), u != u, v != v);\n"
        "  return 0;\n"
        "}\n")
    libdir = os.path.dirname(lib._name)
    exe = tmp_path / "main"
    subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", os.path.join(ROOT, "include"),
                    str(src), "-L", libdir, "-ltree2d_gb300", "-Wl,-rpath," + libdir, "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    assert out == [str(pkg().ERR_NO_TREE), "1", "1"]
