"""The C ABI's structs as the two bindings see them: field offsets and sizes
of include/sphgrid.h (measured by compiling a probe with the host C compiler)
against the ctypes mirror in _lib.py and against the Julia structs of the
ccall shim (julia/SPHtoGridGB300.jl, parsed: no Julia here).  A field that
drifts in one binding shows up here, without a GPU and without Julia.
"""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "sphgrid.h")
JULIA = os.path.join(ROOT, "sphtogrid.jl_gb300", "julia", "SPHtoGridGB300.jl")

# C struct -> (ctypes class in _lib, Julia struct name or None)
STRUCTS = {
    "sphg_params": ("SphgParams", "SphgParams"),
    "sphg_particles": ("SphgParticles", "SphgParticles"),
    "sphg_options": ("SphgOptions", "SphgOptions"),
    "sphg_stats": ("SphgStats", "SphgStats"),
    "sphg_grads": ("SphgGrads", "SphgGrads"),
    "sphg_projection": ("SphgProjection", "SphgProjection"),
    "sphg_healpix_params": ("SphgHealpixParams", None),
}


def _c_fields():
    """{struct: [field, ...]} from the header's typedefs."""
    text = open(HEADER).read()
    out = {}
    for name in STRUCTS:
        m = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), text, re.S)
        assert m, name
        body = re.sub(r"/\*.*?\*/", "", m.group(1), flags=re.S)
        fields = []
        for decl in body.split(";"):
            decl = decl.strip()
            if not decl:
                continue
            names = decl.split(None, 1)[1] if not decl.startswith("const ") else decl.split(None, 2)[2]
            for part in names.split(","):
                part = part.strip().lstrip("*").strip()
                fields.append(re.sub(r"\[.*\]", "", part).strip())
        out[name] = fields
    return out


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no host C compiler")
    fields = _c_fields()
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "%s"' % HEADER, "int main(void) {"]
    for s, fs in fields.items():
        lines.append('  printf("%s sizeof %%zu\\n", sizeof(%s));' % (s, s))
        for f in fs:
            lines.append('  printf("%s %s %%zu\\n", offsetof(%s, %s));' % (s, f, s, f))
    lines += ["  return 0;", "}"]
    d = tmp_path_factory.mktemp("layout")
    src, exe = d / "probe.c", d / "probe"
    src.write_text("\n".join(lines) + "\n")
    subprocess.check_call([cc, "-std=c11", "-o", str(exe), str(src)])
    out = {}
    for ln in subprocess.check_output([str(exe)], text=True).splitlines():
        s, f, v = ln.split()
        out.setdefault(s, {})[f] = int(v)
    return out


def test_ctypes_mirror_matches_header(pkg, c_layout):
    from sphtogrid_gb300 import _lib as L
    for s, (py, _) in STRUCTS.items():
        cls = getattr(L, py)
        assert C_sizeof(cls) == c_layout[s]["sizeof"], s
        for f, off in c_layout[s].items():
            if f == "sizeof":
                continue
            assert getattr(cls, f).offset == off, (s, f)


def C_sizeof(cls):
    import ctypes
    return ctypes.sizeof(cls)


_JL_SIZE = {"Int32": 4, "Int64": 8, "Float32": 4, "Float64": 8, "Cint": 4, "Ptr{Cvoid}": 8}


def _julia_structs():
    text = open(JULIA).read()
    structs = {}
    for m in re.finditer(r"^(?:mutable )?struct (\w+)\n(.*?)^end", text, re.S | re.M):
        fields = []
        for ln in m.group(2).splitlines():
            ln = ln.split("#")[0].strip()
            fm = re.match(r"^(\w+)::(.+)$", ln)
            if fm:
                fields.append((fm.group(1), fm.group(2).strip()))
        structs[m.group(1)] = fields
    return structs


def _jl_layout(structs, name):
    """(size, align, {field: offset}) with C alignment rules (isbits
    structs are laid out as C structs)."""

    def size_align(t):
        if t in _JL_SIZE:
            return _JL_SIZE[t], _JL_SIZE[t]
        tm = re.match(r"NTuple\{(\d+),\s*(\w+(?:\{\w+\})?)\}", t)
        if tm:
            sz, al = size_align(tm.group(2))
            return int(tm.group(1)) * sz, al
        if t in structs:
            sz, al, _ = _jl_layout(structs, t)
            return sz, al
        raise AssertionError(f"unknown Julia field type {t}")

    off, align, offs = 0, 1, {}
    for f, t in structs[name]:
        sz, al = size_align(t)
        off = (off + al - 1) // al * al
        offs[f] = off
        off += sz
        align = max(align, al)
    return (off + align - 1) // align * align, align, offs


def test_julia_structs_match_header(c_layout):
    structs = _julia_structs()
    for s, (_, jl) in STRUCTS.items():
        if jl is None:
            continue
        assert jl in structs, jl
        size, _, offs = _jl_layout(structs, jl)
        assert size == c_layout[s]["sizeof"], s
        c_fields = [f for f in c_layout[s] if f != "sizeof"]
        assert list(offs) == c_fields, (s, list(offs), c_fields)
        for f in c_fields:
            assert offs[f] == c_layout[s][f], (s, f)
