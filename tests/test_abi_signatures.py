"""The C ABI's prototypes (include/simmd.h) against its two bindings, with
no GPU: every ctypes signature of simulationcode_gb300/_lib.py and every
`ccall` of the Julia module (julia/SimulationCodeGPU.jl) and of the binding
examples passes as many arguments as the prototype takes,
with the same scalar types (pointers: any pointer type), and reads the same
return type.  A width mismatch (int32_t vs int64_t, float vs double) would
otherwise pass silently through a C call."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

C_SCALARS = {"int": "i32", "int32_t": "i32", "int64_t": "i64", "uint64_t": "u64", "double": "f64",
             "float": "f32", "void": "void"}


def _c_kind(decl):
    """kind of one C parameter or return type: 'ptr' or a scalar kind"""
    decl = decl.replace("const", " ").strip()
    if "*" in decl:
        return "ptr"
    base = decl.split()[0]
    return C_SCALARS[base]


def header_prototypes():
    src = open(os.path.join(ROOT, "include", "simmd.h")).read()
    src = re.sub(r"/\*.*?\*/", " ", src, flags=re.S)
    src = re.sub(r"//[^\n]*", " ", src)
    protos = {}
    for ret, name, args in re.findall(r"([A-Za-z_][\w\s\*]*?)\b(simmd_\w+)\s*\(([^)]*)\)\s*;", src):
        ret = ret.strip().split("\n")[-1].strip()
        args = args.strip()
        kinds = [] if args in ("", "void") else [_c_kind(a) for a in args.split(",")]
        protos[name] = (_c_kind(ret), kinds)
    return protos


def _ctypes_kind(t):
    if t is None:
        return "void"
    if t in (C.c_void_p, C.c_char_p) or (isinstance(t, type) and issubclass(t, C._Pointer)):
        return "ptr"
    return {C.c_int: "i32", C.c_int32: "i32", C.c_int64: "i64", C.c_uint64: "u64", C.c_double: "f64",
            C.c_float: "f32"}[t]


JULIA_SCALARS = {"Cint": "i32", "Int32": "i32", "Int64": "i64", "UInt64": "u64", "Float64": "f64",
                 "Cdouble": "f64", "Cfloat": "f32", "Float32": "f32", "Cvoid": "void", "Nothing": "void"}


def _julia_kind(t):
    t = t.strip()
    if t.startswith(("Ptr{", "Ref{", "CuPtr{")) or t in ("Cstring",):
        return "ptr"
    return JULIA_SCALARS[t]


def julia_ccalls(path):
    src = open(path).read()
    calls = []
    for name, ret, args in re.findall(r"ccall\(\(:(simmd_\w+),\s*libsimmd\),\s*([\w{}]+),\s*\(([^()]*)\)", src,
                                      flags=re.S):
        parts = [a for a in (x.strip() for x in args.split(",")) if a]
        calls.append((name, _julia_kind(ret), [_julia_kind(a) for a in parts]))
    return calls


def test_header_parses():
    protos = header_prototypes()
    assert protos["simmd_step"] == ("i32", ["ptr", "i64", "ptr"])
    assert protos["simmd_version"] == ("ptr", [])
    assert protos["simmd_transfer_layout"] == ("i64", ["ptr", "i32", "ptr"])
    from test_capi import declared_symbols
    assert sorted(protos) == declared_symbols()


def test_ctypes_signatures_match_the_header():
    from simulationcode_gb300 import _lib
    protos = header_prototypes()
    bad = []
    for name, (res, args) in _lib.SIGNATURES.items():
        want = protos[name]
        got = (_ctypes_kind(res), [_ctypes_kind(a) for a in args])
        if got != want:
            bad.append((name, got, want))
    assert not bad, bad


@pytest.mark.parametrize("path", ["julia/SimulationCodeGPU.jl", "INTEGRATION.md"])
def test_julia_ccalls_match_the_header(path):
    protos = header_prototypes()
    calls = julia_ccalls(os.path.join(ROOT, path))
    assert len(calls) >= (25 if path.endswith(".jl") else 8)
    bad = [(n, r, a, protos.get(n)) for n, r, a in calls if protos.get(n) != (r, a)]
    assert not bad, bad


def header_struct(name):
    """[(field, kind)] of `typedef struct name { ... } name;` in the header"""
    src = open(os.path.join(ROOT, "include", "simmd.h")).read()
    src = re.sub(r"/\*.*?\*/", " ", src, flags=re.S)
    body = re.search(r"typedef struct %s\s*\{(.*?)\}\s*%s;" % (name, name), src, flags=re.S).group(1)
    fields = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        typ, names = decl.split(None, 1)
        fields += [(n.strip(), C_SCALARS[typ]) for n in names.split(",")]
    return fields


def julia_struct(name, path="julia/SimulationCodeGPU.jl"):
    src = open(os.path.join(ROOT, path)).read()
    body = re.search(r"\nstruct %s[^\n]*\n(.*?)\nend" % name, src, flags=re.S).group(1)
    fields = []
    for decl in re.split(r"[;\n]", body):
        decl = decl.strip()
        if decl:
            n, t = decl.split("::")
            fields.append((n.strip(), JULIA_SCALARS[t.strip()]))
    return fields


@pytest.mark.parametrize("cname,pyname,jlname", [("simmd_params", "Params", "SimmdParams"),
                                                 ("simmd_stats", "Stats", "SimmdStats")])
def test_structs_match_the_header(cname, pyname, jlname):
    """the parameter and statistics structs: the same fields, in the same
    order, of the same widths in the header, the ctypes mirror and the Julia
    module (isbits structs laid out as C's)"""
    from simulationcode_gb300 import _lib
    want = header_struct(cname)
    py = [(n, _ctypes_kind(t)) for n, t in getattr(_lib, pyname)._fields_]
    assert py == want
    assert julia_struct(jlname) == want
    if cname == "simmd_params":  # the copy in the binding examples
        assert julia_struct(jlname, "INTEGRATION.md") == want
