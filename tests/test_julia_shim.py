"""Static consistency of the Julia drop-in (itensors.jl_gb300/julia/NDTensorsGB300Ext.jl)
with the C ABI: every entry point it ccalls is declared in include/ndtensors_gb300.h and
exported by the built library, with as many arguments as the declaration has.  (No Julia
toolchain is available to run the shim itself.)"""
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
SHIM = ROOT / "itensors.jl_gb300" / "julia" / "NDTensorsGB300Ext.jl"
HEADER = ROOT / "include" / "ndtensors_gb300.h"


def _split_top(s):
    """Split on commas outside brackets/braces/parens."""
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
    return [x.strip() for x in out]


def _balanced(text, start):
    """Text of the parenthesised group opening at text[start] == '('."""
    depth = 0
    for i in range(start, len(text)):
        if text[i] == "(":
            depth += 1
        elif text[i] == ")":
            depth -= 1
            if depth == 0:
                return text[start + 1:i]
    raise ValueError("unbalanced")


def _shim_calls():
    src = SHIM.read_text()
    calls = []
    for m in re.finditer(r"ccall\(\(:(\w+), LIB\),", src):
        rest = src[m.end():]
        # return type, then the argument-type tuple
        k = rest.index("(")
        types = _split_top(_balanced(rest, k))
        calls.append((m.group(1), len(types)))
    return calls


def _header_arity():
    hdr = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    ar = {}
    for m in re.finditer(r"\b(?:nd_status|const char\s*\*|int32_t|void)\s*(nd_\w+)\s*\(", hdr):
        params = _balanced(hdr, m.end() - 1).strip()
        ar[m.group(1)] = 0 if params in ("", "void") else len(_split_top(params))
    return ar


def test_shim_calls_match_header():
    calls = _shim_calls()
    assert len(calls) >= 20
    ar = _header_arity()
    for name, n in calls:
        assert name in ar, f"{name} is not declared in the header"
        assert ar[name] == n, f"{name}: shim passes {n} argument types, header declares {ar[name]}"


def test_shim_symbols_exported():
    import ctypes
    lib_path = ROOT / "itensors.jl_gb300" / "ndtensors_gb300" / "libndtensors_gb300.so"
    if not lib_path.exists():
        pytest.skip("library not built")
    try:
        lib = ctypes.CDLL(str(lib_path))
    except OSError as e:
        pytest.skip(f"library does not load here: {e}")
    for name, _ in _shim_calls():
        assert hasattr(lib, name), f"{name} not exported"
