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


# the reference's generic functions on the hot path: positional arity and the
# position (1-based) of the neighbour-list argument, from their definitions
REFERENCE_GENERICS = {
    "update_neighbor_lists!": (4, 4),        # src/NeighborLists.jl:24
    "calculate_new_forces!": (3, 3),         # src/MD.jl:262
    "do_time_step": (5, 4),                  # src/MD.jl:429, 499
    "run_short_MD_equilibration!": (4, 4),   # src/MD.jl:579
    "calculate_full_energy": (3, 3),         # src/AuxiliaryFunctions.jl:22
    "compute_potential_energy!": (4, 4),     # src/AuxiliaryFunctions.jl:186
    "print_log_data": (5, 4),                # src/MD.jl:610
    "find_inherent_structure": (5, 4),       # src/InherentStructure.jl:5
    "do_MC_step!": (5, 4),                   # src/MC.jl:139
}


def _split_args(s):
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch in "({[":
            depth += 1
        elif ch in ")}]":
            depth -= 1
        if ch == "," and depth == 0:
            out.append(cur)
            cur = ""
        else:
            cur += ch
    if cur.strip():
        out.append(cur)
    return [a.strip() for a in out]


def test_julia_methods_extend_the_reference_generics():
    """every hot-path generic function of the reference gets a method for the
    device neighbour list with the reference's positional arity and the list
    in the reference's position, and the module imports the name from
    SimulationCode (so the method extends the reference's function, which
    the reference's own driver then dispatches to)"""
    src = open(os.path.join(ROOT, "julia", "SimulationCodeGPU.jl")).read()
    imports = re.search(r"import SimulationCode:(.*?)\n\s*using", src, flags=re.S).group(1)
    imported = {x.strip() for x in imports.replace("\n", " ").split(",")}
    found = {}
    for name, args in re.findall(r"(?:^function |^)([A-Za-z_!]+)\(([^;)]*(?:\([^)]*\)[^;)]*)*)[;)]", src,
                                 flags=re.M):
        parts = _split_args(args)
        pos = [k + 1 for k, a in enumerate(parts) if a.endswith("::GPUNeighborList")]
        if pos:
            found.setdefault(name, set()).add((len(parts), pos[0]))
    for name, sig in REFERENCE_GENERICS.items():
        assert name in imported, name
        assert sig in found.get(name, set()), (name, found.get(name))
    # initialize_neighbor_struct(skin, box_size, force_cutoff, N, D_array, dims;
    # maxneighbours) (src/DataStructs.jl:349) plus the trailing device marker
    assert "initialize_neighbor_struct" in imported
    assert re.search(r"function initialize_neighbor_struct\(skin_distance, box_size, force_cutoff, N, D_array, dims, "
                     r"dev::GPU;", src)
