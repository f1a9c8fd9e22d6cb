"""The Julia binding (hssmatrices.jl_gb300/julia/HssGpu.jl) against include/hssgpu.h (CPU).

Julia is not installed here, so the shim cannot run; instead every
``ccall((:name, lib), Ret, (Args...), ...)`` in it is parsed and its return and
argument types are checked, position by position, against the prototype of
``name`` in the C header, and the library is checked to export ``name``.
"""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHIM = os.path.join(ROOT, "hssmatrices.jl_gb300", "julia", "HssGpu.jl")
HEADER = os.path.join(ROOT, "include", "hssgpu.h")

# Julia ccall types -> the C type classes they may bind
JULIA_TO_C = {
    "Cint": {"int"},
    "Int32": {"int32_t"},
    "Int64": {"int64_t"},
    "Float64": {"double"},
    "Cstring": {"const char*"},
    "Ptr{Cvoid}": {"hss_handle", "hss_factor", "void*"},
    "Ptr{Float64}": {"double*", "const double*"},
    "Ptr{Int64}": {"int64_t*", "const int64_t*"},
    "Ref{Ptr{Cvoid}}": {"hss_handle*", "hss_factor*"},
    "Ref{Int64}": {"int64_t*"},
    "Ref{SolveStats}": {"hss_solve_stats*"},
}


def _split_top(s):
    """Split on commas outside braces/parentheses."""
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch in "({":
            depth += 1
        elif ch in ")}":
            depth -= 1
        if ch == "," and depth == 0:
            out.append(cur.strip())
            cur = ""
        else:
            cur += ch
    if cur.strip():
        out.append(cur.strip())
    return out


def shim_calls():
    src = open(SHIM).read()
    calls = []
    for m in re.finditer(r"ccall\(\(:(\w+),\s*lib\),", src):
        i = m.end()
        depth, j = 1, i   # inside ccall(
        while depth:
            depth += {"(": 1, ")": -1}.get(src[j], 0)
            j += 1
        args = _split_top(src[i:j - 1])
        ret, argtypes = args[0], args[1]
        assert argtypes.startswith("(") and argtypes.endswith(")"), argtypes
        tys = _split_top(argtypes[1:-1])
        calls.append((m.group(1), ret, tys))
    return calls


def header_protos():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    protos = {}
    for m in re.finditer(r"\b(int|int64_t|int32_t|const char\*)\s+(hss_\w+)\s*\(([^)]*)\);", txt):
        params = [p.strip() for p in m.group(3).split(",") if p.strip() and p.strip() != "void"]
        types = []
        for p in params:
            p = re.sub(r"\s+", " ", p)
            name_m = re.match(r"(.*?)(\w+)$", p)
            ty = name_m.group(1).replace(" *", "*").strip()
            ty = re.sub(r"\s*\*\s*", "*", ty)
            types.append(ty)
        protos[m.group(2)] = (m.group(1), types)
    return protos


def test_shim_is_present_and_parsed():
    calls = shim_calls()
    names = {c[0] for c in calls}
    for need in ("hss_create", "hss_destroy", "hss_matmul_host", "hss_ulvfactsolve_host", "hss_ulvfactor",
                 "hss_ulvsolve_host", "hss_factor_destroy", "hss_last_error", "hss_set_option", "hss_ldiv",
                 "hss_rdiv", "hss_transpose", "hss_size"):
        assert need in names, need


@pytest.mark.parametrize("call", shim_calls(), ids=lambda c: c[0])
def test_ccall_matches_header(call):
    name, ret, tys = call
    protos = header_protos()
    assert name in protos, f"{name} is not declared in include/hssgpu.h"
    cret, ctys = protos[name]
    assert cret in JULIA_TO_C[ret] or (ret == "Cint" and cret == "int"), (name, ret, cret)
    assert len(tys) == len(ctys), (name, tys, ctys)
    for k, (jt, ct) in enumerate(zip(tys, ctys)):
        assert jt in JULIA_TO_C, (name, k, jt)
        assert ct in JULIA_TO_C[jt], f"{name} argument {k}: Julia {jt} vs C {ct}"


def test_library_exports_shim_symbols(pkg):
    lib = pkg._lib.load()
    for name, _ret, _tys in shim_calls():
        assert hasattr(lib, name), name
