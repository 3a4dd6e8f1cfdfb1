"""The bindings against include/madsdp_gpu.h, read as source:

* the Julia struct mirrors (madsdp.jl_gb300/julia/MadSDPGPU.jl) have the
  fields, order and widths of the ctypes mirrors, whose layouts
  tests/test_abi.py checks against the C compiler;
* every Julia ccall and every entry of the ctypes signature table
  (madsdp_gpu._lib.SIGNATURES) passes the header's argument kinds
  (pointer, 32-bit or 64-bit integer, double) in the header's order.

Julia is not in this image, so its side is checked from the source."""
import ctypes as C
import os
import re

import pytest

from madsdp_gpu import _lib

JL = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "madsdp.jl_gb300", "julia",
                  "MadSDPGPU.jl")


def julia_structs():
    src = open(JL).read()
    out = {}
    for name, body in re.findall(r"^struct (\w+)\n(.*?)^end", src, flags=re.S | re.M):
        fields = re.findall(r"(\w+)::([\w{}]+)", body)
        out[name] = fields
    return out


def kind(t):
    if isinstance(t, str):
        return "ptr" if t.startswith("Ptr{") else {"Int32": "i32", "Int64": "i64", "Float64": "f64"}[t]
    if t is C.c_int32:
        return "i32"
    if t is C.c_int64:
        return "i64"
    if t is C.c_double:
        return "f64"
    if issubclass(t, C._Pointer) or t is C.c_void_p:
        return "ptr"
    raise TypeError(t)


@pytest.mark.parametrize("name", ["Components", "Options", "ProblemDesc", "Stats"])
def test_struct_mirrors(name):
    jl = julia_structs()[name]
    py = getattr(_lib, name)._fields_
    assert [f for f, _ in jl] == [f for f, _ in py]
    assert [kind(t) for _, t in jl] == [kind(t) for _, t in py]


HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "madsdp_gpu.h")


def split_top(s):
    """Split on commas outside (), {} and []."""
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch in "({[":
            depth += 1
        elif ch in ")}]":
            depth -= 1
        if ch == "," and depth == 0:
            out.append(cur.strip())
            cur = ""
        else:
            cur += ch
    if cur.strip():
        out.append(cur.strip())
    return out


def balanced(s, i):
    """The text inside the parenthesis opening at s[i]."""
    depth = 0
    for j in range(i, len(s)):
        depth += s[j] == "("
        depth -= s[j] == ")"
        if depth == 0:
            return s[i + 1:j]
    raise ValueError("unbalanced")


def julia_ccalls():
    src = open(JL).read()
    calls = {}
    for m in re.finditer(r"ccall\(\(:(\w+), LIB\),", src):
        rest = src[m.end():]
        ret, after = rest.split(",", 1)
        i = after.index("(")
        args = split_top(balanced(after, i))
        calls.setdefault(m.group(1), []).append((ret.strip(), args))
    return calls


def header_functions():
    src = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    out = {}
    for m in re.finditer(r"\b(\w[\w\s\*]*?)\b(msdp_\w+)\s*\(([^;{]*?)\)\s*;", src, flags=re.S):
        params = [p.strip() for p in split_top(m.group(3)) if p.strip() and p.strip() != "void"]
        out[m.group(2)] = params
    return out


def jl_kind(t):
    t = t.strip()
    if t.startswith(("Ptr{", "Ref{")) or t == "Cstring":
        return "ptr"
    return {"Cint": "i32", "Int32": "i32", "Int64": "i64", "Float64": "f64", "Cdouble": "f64"}[t]


def c_kind(p):
    if "*" in p:
        return "ptr"
    ty = p.rsplit(None, 1)[0] if " " in p else p
    return {"int": "i32", "int32_t": "i32", "int64_t": "i64", "double": "f64"}[ty.replace("const ", "").strip()]


def test_ccall_signatures_match_header():
    hdr = header_functions()
    calls = julia_ccalls()
    assert len(calls) >= 10
    for name, uses in calls.items():
        assert name in hdr, name
        for ret, args in uses:
            assert [jl_kind(a) for a in args] == [c_kind(p) for p in hdr[name]], (name, args, hdr[name])


def py_kind(t):
    if t is C.c_int or t is C.c_int32:
        return "i32"
    if t is C.c_int64:
        return "i64"
    if t is C.c_double:
        return "f64"
    if t in (C.c_void_p, C.c_char_p) or issubclass(t, C._Pointer):
        return "ptr"
    raise TypeError(t)


def test_python_signatures_match_header():
    """The ctypes table of madsdp_gpu._lib declares every header function
    with the header's argument kinds."""
    hdr = header_functions()
    sigs = {name: args for name, _, args in _lib.SIGNATURES}
    assert set(sigs) == set(hdr)
    for name, args in sigs.items():
        assert [py_kind(a) for a in args] == [c_kind(p) for p in hdr[name]], (name, args, hdr[name])
