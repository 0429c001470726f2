"""The ctypes binding against the C header, without a GPU.

A drift between include/gstools_core_gb300.h and the Python binding
(gstools_core/_native.py) would pass wrong arguments through the C ABI.
Checked here: every prototype's return and parameter types against the
binding's restype/argtypes, and every public struct's size and field
offsets, as a C compiler lays them out (gcc on the header), against the
ctypes structures.
"""
import ctypes
import os
import re
import shutil
import subprocess

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "gstools_core_gb300.h")


def _prototypes():
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    out = {}
    for ret, name, params in re.findall(r"^([A-Za-z_][\w \*]*?)\s*\b(gsc_\w+)\s*\(([^)]*)\)\s*;",
                                        text, flags=re.M):
        ps = [p.strip() for p in params.replace("\n", " ").split(",")]
        out[name] = (ret.strip(), [] if ps in ([""], ["void"]) else ps)
    return out


def _c_kind(decl: str) -> str:
    """Kind of a C parameter or return type ('name' stripped)."""
    decl = re.sub(r"\bconst\b", "", decl).strip()
    if "*" in decl:
        base = decl.split("*")[0].split()[-1]
        stars = decl.count("*")
        if base == "char" and stars == 1:
            return "char*"
        if stars == 1 and base in ("gsc_opts", "gsc_batch_item", "gsc_batch_config",
                                   "gsc_sample_item"):
            return base + "*"
        return "ptr"
    base = decl.split()[0]
    return {"int": "i32", "int32_t": "i32", "int64_t": "i64", "uint64_t": "u64",
            "double": "f64"}[base]


def _py_kind(t) -> str:
    from gstools_core import _native as n
    if t is None:
        return "void"
    for ctype, kind in ((ctypes.c_char_p, "char*"), (ctypes.c_void_p, "ptr"),
                        (ctypes.c_int64, "i64"), (ctypes.c_uint64, "u64"),
                        (ctypes.c_int32, "i32"), (ctypes.c_double, "f64")):
        if t is ctype:
            return kind
    structs = {n.GscOpts: "gsc_opts*", n.GscBatchItem: "gsc_batch_item*",
               n.GscBatchConfig: "gsc_batch_config*", n.GscSampleItem: "gsc_sample_item*"}
    if hasattr(t, "_type_") and t._type_ in structs:
        return structs[t._type_]
    if hasattr(t, "_type_"):
        return "ptr"                       # POINTER(scalar) or POINTER(c_void_p)
    raise AssertionError(f"unmapped ctypes type {t}")


def test_prototypes_match_the_binding(gsc):
    from gstools_core import _native
    protos = _prototypes()
    assert set(protos) == set(_native.SIGNATURES)
    for name, (ret, params) in protos.items():
        res, args = _native.SIGNATURES[name]
        assert _c_kind(ret) == _py_kind(res), name
        c_kinds = [_c_kind(re.sub(r"\s*\b\w+\s*$", "", p) if not p.endswith("*") else p)
                   for p in params]
        assert c_kinds == [_py_kind(a) for a in args], name


_STRUCTS = {
    "gsc_opts": "GscOpts",
    "gsc_batch_item": "GscBatchItem",
    "gsc_batch_config": "GscBatchConfig",
    "gsc_sample_item": "GscSampleItem",
}


def _c_layout(tmp_path):
    gcc = shutil.which("gcc") or shutil.which("cc")
    if gcc is None:
        pytest.skip("no C compiler")
    from gstools_core import _native
    lines = ['#include <stddef.h>', '#include <stdio.h>', f'#include "{HEADER}"', "int main(void) {"]
    for cname, pyname in _STRUCTS.items():
        st = getattr(_native, pyname)
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for field, _ in st._fields_:
            lines.append(f'printf("{cname} {field} %zu\\n", offsetof({cname}, {field}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([gcc, "-std=c99", str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return {tuple(l.split()[:2]): int(l.split()[2]) for l in out.splitlines()}


def test_struct_layouts_match_the_binding(gsc, tmp_path):
    from gstools_core import _native
    c = _c_layout(tmp_path)
    for cname, pyname in _STRUCTS.items():
        st = getattr(_native, pyname)
        assert c[(cname, "size")] == ctypes.sizeof(st), cname
        for field, _ in st._fields_:
            assert c[(cname, field)] == getattr(st, field).offset, (cname, field)


def test_batch_item_numpy_layout_matches_the_struct():
    """summate_batch fills its items through a numpy structured type; it must
    have the C struct's size and field offsets."""
    n = pytest.importorskip("gstools_core._native")
    dt = n.BATCH_ITEM_DTYPE
    assert dt.itemsize == ctypes.sizeof(n.GscBatchItem)
    for name, _ in n.GscBatchItem._fields_:
        assert dt.fields[name][1] == getattr(n.GscBatchItem, name).offset, name
