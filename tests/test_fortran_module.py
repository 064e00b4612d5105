"""The Fortran binding module include/m_tree_bindc.f90 against the C header
and the library, without a Fortran compiler: every bind(c) procedure names
an exported function declared in include/tree2d.h with as many arguments,
each argument passed by value in Fortran is a scalar in C and each one passed
by reference a pointer, and a function returns a C int where the module says
integer(c_int) (a subroutine: void).  make_tree and biot_tree keep the
reference's interface (ver-c/src/m_tree_bindc.f90:1-17): nvor_b, x and y by
value, the arrays and u, v by reference."""
from __future__ import annotations

import os
import re

from conftest import ROOT

MODULE = os.path.join(ROOT, "include", "m_tree_bindc.f90")
HEADER = os.path.join(ROOT, "include", "tree2d.h")


def fortran_procedures():
    src = open(MODULE).read()
    src = re.sub(r"!.*", "", src)
    out = {}
    pat = re.compile(r"(subroutine|integer\(c_int\)\s+function)\s+(\w+)\s*\(([^)]*)\)\s*bind\(c,\s*name=\"(\w+)\"\)(.*?)end\s+(?:subroutine|function)",
                     re.S | re.I)
    for kind, name, args, cname, body in pat.findall(src):
        args = [a.strip().lower() for a in args.split(",") if a.strip()]
        by_value = set()
        for line in body.splitlines():
            if "::" not in line:
                continue
            attrs, names = line.split("::", 1)
            names = [n.split("(")[0].strip().lower() for n in re.split(r",(?![^()]*\))", names)]
            if re.search(r"\bvalue\b", attrs, re.I):
                by_value.update(names)
        out[cname] = ("void" if kind.lower() == "subroutine" else "int", args, by_value)
    return out


def c_prototypes():
    src = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    protos = {}
    for ret, name, params in re.findall(r"\b(void|int|double|const char\s*\*)\s+(\w+)\s*\(([^)]*)\)\s*;", src):
        ps = [] if params.strip() in ("", "void") else [p.strip() for p in params.split(",")]
        protos[name] = (ret.replace(" ", ""), ps)
    return protos


def test_module_matches_header_and_library(lib):
    procs = fortran_procedures()
    assert {"make_tree", "biot_tree", "biot_tree_batch", "tree2d_learn_load"} <= set(procs)
    protos = c_prototypes()
    for cname, (ret, args, by_value) in procs.items():
        assert hasattr(lib, cname), cname
        assert cname in protos, cname
        cret, cparams = protos[cname]
        assert cret == ret, (cname, cret, ret)
        assert len(cparams) == len(args), (cname, cparams, args)
        for a, cp in zip(args, cparams):
            assert ("*" in cp) == (a not in by_value), (cname, a, cp)


def test_reference_interface_kept():
    procs = fortran_procedures()
    assert procs["make_tree"][1] == ["nvor_b", "vor_b", "cir_b", "cor_b"]
    assert procs["make_tree"][2] == {"nvor_b"}
    assert procs["biot_tree"][1] == ["x", "y", "u", "v"]
    assert procs["biot_tree"][2] == {"x", "y"}
