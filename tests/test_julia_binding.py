"""CPU checks of the Julia binding julia/HT3D.jl against the C header and the
ctypes mirror: the file is what julia/generate.py writes today; every header
prototype has a `ccall` with the same symbol, arity and C-compatible argument
types; every parameter struct has the ctypes mirror's fields in the same
order and types; every reference kernel the header names has a drop-in
wrapper.  (No Julia is run: there is none here.)"""
import ctypes
import os
import re
import sys

import pytest

from hydrothermal3d_gb300 import _lib, abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
JL = os.path.join(ROOT, "julia", "HT3D.jl")
HEADER = os.path.join(ROOT, "include", "ht3d.h")


@pytest.fixture(scope="module")
def jl():
    with open(JL) as f:
        return f.read()


@pytest.fixture(scope="module")
def gen():
    sys.path.insert(0, os.path.join(ROOT, "julia"))
    try:
        import generate
    finally:
        sys.path.pop(0)
    return generate


def _split_top(s):
    """Split a Julia type tuple body on top-level commas."""
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch == "{":
            depth += 1
        elif ch == "}":
            depth -= 1
        if ch == "," and depth == 0:
            out.append(cur.strip())
            cur = ""
        else:
            cur += ch
    if cur.strip():
        out.append(cur.strip())
    return out


def _ccalls(text):
    res = {}
    for m in re.finditer(r"ccall\(\(:(ht3d_\w+), libht3d\), (\w+), \((.*?)\)(?:, |\))", text):
        body = m.group(3)
        res[m.group(1)] = (m.group(2), _split_top(body))
    return res


# C type -> Julia types a ccall may declare for it (device arrays as CuPtr,
# host arrays as Ptr; structs by Ref or Ptr)
def _allowed(ctype):
    base = ctype.replace("const ", "").strip()
    table = {
        "double": {"Cdouble"}, "int": {"Cint"}, "long long": {"Clonglong"},
        "unsigned long long": {"Culonglong"}, "double*": {"CuPtr{Cdouble}", "Ptr{Cdouble}"},
        "float*": {"CuPtr{Cfloat}"}, "int*": {"Ptr{Cint}"}, "unsigned long long*": {"Ptr{Culonglong}"},
        "void*": {"Ptr{Cvoid}"}, "char*": {"Cstring"}, "char* const*": {"Ptr{Cstring}"},
        "double* const*": {"Ptr{Ptr{Cdouble}}"}, "ht3d_ctx*": {"Ptr{Cvoid}"}, "ht3d_ctx**": {"Ref{Ptr{Cvoid}}"},
    }
    if base in table:
        return table[base]
    m = re.match(r"ht3d_(\w+)\*$", base)
    assert m, ctype
    jname = {"dyrel_params": "DyrelParams", "dyrel_stats": "DyrelStats", "hrl_params": "HrlParams",
             "v18_params": "V18Params", "khaled_geom": "KhaledGeom", "post_params": "PostParams",
             "post_fields": "PostFields", "instance": "Instance"}[m.group(1)]
    return {f"Ref{{{jname}}}", f"Ptr{{{jname}}}"}


def test_binding_is_up_to_date(jl, gen):
    assert jl == gen.generate(), "julia/HT3D.jl is stale: run python julia/generate.py"


def test_every_prototype_has_a_matching_ccall(jl, gen):
    calls = _ccalls(jl)
    protos = gen.parse_header()
    assert {n for _, n, _ in protos} == set(calls)
    assert set(calls) == set(_lib.parse_header())
    ret_map = {"int": "Cint", "const char*": "Cstring", "unsigned long long": "Culonglong", "double": "Cdouble"}
    for ret, name, params in protos:
        jret, jtypes = calls[name]
        assert jret == ret_map[ret], name
        assert len(jtypes) == len(params), name
        for (ctype, pname), jt in zip(params, jtypes):
            assert jt in _allowed(ctype), (name, pname, ctype, jt)


def test_device_and_host_pointers(jl):
    """Host-side outputs are Ptr, device arrays CuPtr (CUDA.jl converts a CuArray only to CuPtr)."""
    calls = _ccalls(jl)
    assert calls["ht3d_reduce"][1][-1] == "Ptr{Cdouble}"
    assert calls["ht3d_Nusselt"][1][-1] == "Ptr{Cdouble}"
    assert calls["ht3d_ComputeFlux"][1][1] == "CuPtr{Cdouble}"
    assert calls["ht3d_dyrel_iterate"][1][12:14] == ["Ptr{Cint}", "Ptr{Cdouble}"]  # BC types, values
    assert calls["ht3d_weno5_advect_f32"][1][1] == "CuPtr{Cfloat}"


def _jl_structs(text):
    res = {}
    for m in re.finditer(r"Base\.@kwdef struct (\w+)\n(.*?)\nend", text, re.S):
        fields = []
        for line in m.group(2).splitlines():
            fm = re.match(r"\s+(\w+)::(.+?) = ", line)
            if fm:
                fields.append((fm.group(1), fm.group(2)))
        res[m.group(1)] = fields
    return res


def _ctypes_to_jl(t):
    if t is ctypes.c_double:
        return "Cdouble"
    if t is ctypes.c_int:
        return "Cint"
    if t is ctypes.c_void_p:
        return "CuPtr{Cdouble}"
    if issubclass(t, ctypes.Array):
        return f"NTuple{{{t._length_}, {_ctypes_to_jl(t._type_)}}}"
    if issubclass(t, ctypes._Pointer):
        return f"Ptr{{{t._type_.__name__}}}"
    return t.__name__


@pytest.mark.parametrize("name", ["DyrelParams", "DyrelStats", "HrlParams", "V18Params", "KhaledGeom", "PostParams",
                                  "PostFields", "Instance"])
def test_structs_mirror_the_ctypes_layout(jl, name):
    js = _jl_structs(jl)[name]
    cls = getattr(abi, name)
    assert [f for f, _ in js] == [f for f, _ in cls._fields_]
    assert [t for _, t in js] == [_ctypes_to_jl(t) for _, t in cls._fields_]


def test_every_reference_kernel_has_a_dropin(jl):
    src = open(HEADER).read()
    toks = re.findall(r"^/\* ([^\s]+)\s+(?:\(dimensional\)\s+)?(?:Dimension|tools|:|kernels_|v1 |\()", src, re.M)
    names = set()
    for t in toks:
        if "/" in t or not re.search(r"[A-Zϕ]", t) or t == "Reductions":
            continue
        parts = [t]
        while any("{" in p for p in parts):  # expand V{x,y,z}PlusMinus! and the like
            nxt = []
            for p in parts:
                m = re.search(r"\{([^}]*)\}", p)
                if not m:
                    nxt.append(p)
                    continue
                nxt += [p[:m.start()] + alt + p[m.end():] for alt in m.group(1).split(",")]
            parts = nxt
        names.update(parts)
    assert len(names) >= 55
    defined = set(re.findall(r"^function ([^\s(]+)\(", jl, re.M))
    missing = [n for n in sorted(names) if n not in defined and n + "!" not in defined]
    assert not missing, missing


def test_dispatch_by_arity_keeps_both_reference_files_apart(jl):
    """Kernels named alike in the dimensionless and dimensional files (Init_vel!,
    InitThermal!, InitDarcy!, SetPressureBCs!) and the v1/v2 Advect! differ in
    arity, so Julia dispatches each call to the right entry point."""
    for name in ("Init_vel!", "InitThermal!", "InitDarcy!", "SetPressureBCs!", "Advect!"):
        sigs = re.findall(r"^function " + re.escape(name) + r"\(([^;]*);", jl, re.M)
        assert len(sigs) == 2, name
        assert len({len(s.split(",")) for s in sigs}) == 2, name
