"""The Julia ccall layer (diffpumas.jl_gb300/julia/DiffPumasGPU.jl) against the
C header, on the CPU (no Julia toolchain exists on these machines):

- every Julia struct DpFoo that mirrors a C struct dp_foo has the C struct's
  field names in the same order, each with the Julia type of its C type, so
  offsets and sizes agree; the layout computed from the Julia types also
  equals the ctypes layout the Python tests pass through the same ABI;
- every C struct the header defines has its Julia mirror;
- every ccall names a symbol the header declares, and every struct a ccall
  passes by Ref or Ptr is defined in the module.
"""
import ctypes as C
import os
import re

import pytest

from conftest import ROOT

JL = os.path.join(ROOT, "diffpumas.jl_gb300", "julia", "DiffPumasGPU.jl")
HDR = os.path.join(ROOT, "include", "dpgpu.h")

# Julia type of a C field type, and (size, alignment) of each Julia type
C_TO_JL = {"int": "Cint", "double": "Cdouble", "long": "Clong", "uint64_t": "UInt64",
           "const char*": "Cstring", "const double*": "Ptr{Cdouble}",
           "const int32_t*": "Ptr{Int32}", "const int64_t*": "Ptr{Int64}"}
JL_SIZE = {"Cint": (4, 4), "Cdouble": (8, 8), "Clong": (8, 8), "UInt64": (8, 8),
           "Cstring": (8, 8), "Int32": (4, 4), "Int64": (8, 8)}


def camel(cname):
    return "".join(p.capitalize() for p in cname.split("_"))


def c_structs():
    h = re.sub(r"/\*.*?\*/", "", open(HDR).read(), flags=re.S)
    out = {}
    for m in re.finditer(r"typedef struct\s*\{(.*?)\}\s*(\w+);", h, re.S):
        fields = []
        for decl in m.group(1).split(";"):
            decl = " ".join(decl.split())
            if not decl:
                continue
            mm = re.match(r"((?:const )?[\w]+\s*\*?)\s*(.*)", decl)
            base, names = mm.group(1).replace(" *", "*").strip(), mm.group(2)
            if names.startswith("*"):
                base, names = base + "*", names[1:]
            for n in names.split(","):
                n = n.strip()
                if n.startswith("*"):
                    fields.append((n[1:], base + "*"))
                else:
                    fields.append((n, base))
        out[m.group(2)] = fields
    return out


def jl_structs():
    src = open(JL).read()
    out = {}
    for m in re.finditer(r"^struct (\w+)\s*\n?(.*?)\bend\b", src, re.S | re.M):
        body = re.sub(r"#.*", "", m.group(2))
        out[m.group(1)] = re.findall(r"(\w+)::([\w{}]+)", body)
    return out


def jl_type_of(ctype):
    if ctype in C_TO_JL:
        return C_TO_JL[ctype]
    m = re.match(r"(?:const )?(dp_\w+)(\*?)$", ctype)
    assert m, ctype
    return f"Ptr{{{camel(m.group(1))}}}" if m.group(2) else camel(m.group(1))


def layout(jl, name):
    """(size, alignment) of a Julia struct under the C rules."""
    off, align = 0, 1
    for _, t in jl[name]:
        if t.startswith("Ptr{"):
            s, a = 8, 8
        elif t in JL_SIZE:
            s, a = JL_SIZE[t]
        else:
            s, a = layout(jl, t)
        off = (off + a - 1) // a * a + s
        align = max(align, a)
    return (off + align - 1) // align * align, align


def test_every_c_struct_has_its_julia_mirror():
    cs, jl = c_structs(), jl_structs()
    assert len(cs) >= 20
    for cname, fields in cs.items():
        jname = camel(cname)
        assert jname in jl, f"{jname} missing from the Julia module"
        assert [f for f, _ in jl[jname]] == [f for f, _ in fields], jname
        for (f, ct), (_, jt) in zip(fields, jl[jname]):
            assert jt == jl_type_of(ct), f"{jname}.{f}: {jt} for C {ct}"


def test_julia_layouts_equal_the_ctypes_layouts():
    from dpgpu import _lib
    jl = jl_structs()
    checked = 0
    for jname in jl:
        py = getattr(_lib, jname, None)
        if not (isinstance(py, type) and issubclass(py, C.Structure)):
            continue
        assert [f for f, _ in jl[jname]] == [f for f, _ in py._fields_], jname
        assert layout(jl, jname)[0] == C.sizeof(py), jname
        checked += 1
    assert checked >= 10


def test_every_ccall_names_a_declared_symbol():
    src = open(JL).read()
    hdr = open(HDR).read()
    calls = set(re.findall(r"ccall\(\(:(\w+),\s*lib\)", src))
    assert len(calls) >= 25
    for name in calls:
        assert re.search(rf"\b{name}\s*\(", hdr), f"{name} is not declared in dpgpu.h"
    used = set(re.findall(r"(?:Ref|Ptr)\{(Dp\w+)\}", src))
    defined = set(jl_structs())
    assert used <= defined, used - defined


def offsets(jl, name):
    """Field offsets of a Julia struct under the C rules."""
    off, out = 0, []
    for f, t in jl[name]:
        if t.startswith("Ptr{"):
            sz, a = 8, 8
        elif t in JL_SIZE:
            sz, a = JL_SIZE[t]
        else:
            sz, a = layout(jl, t)
        off = (off + a - 1) // a * a
        out.append((f, off))
        off += sz
    return out


def test_layouts_equal_the_c_compilers(tmp_path):
    """Every field offset and every struct size computed from the Julia types
    equals what gcc gives the header's structs (offsetof / sizeof)."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    cs, jl = c_structs(), jl_structs()
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "dpgpu.h"', "int main(void) {"]
    for cname, fields in cs.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for f, _ in fields:
            lines.append(f'  printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.check_call([cc, "-std=c11", "-I", os.path.dirname(HDR), str(src), "-o", str(exe)])
    got = {}
    for line in subprocess.check_output([str(exe)], text=True).splitlines():
        s, f, v = line.split()
        got[(s, f)] = int(v)
    for cname in cs:
        jname = camel(cname)
        assert layout(jl, jname)[0] == got[(cname, "size")], jname
        for f, off in offsets(jl, jname):
            assert off == got[(cname, f)], f"{jname}.{f}"
