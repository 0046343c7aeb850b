"""CPU checks of the Fortran interface module fortran/peps_mg_gpu.f90 against the C-ABI.

No Fortran compiler exists here, so the module is checked as text against the header:
* every entry point of include/peps_mg.h has a bind(C) interface of that name, and the
  module binds nothing the header does not declare;
* each interface has as many dummy arguments as the C prototype has parameters;
* the bind(C) derived types pmg_config_t and pmg_report_t list the C structs' members in
  the same order, and the offsets those interoperable types imply (c_int 4, c_float 4,
  c_double 8, c_ptr 8 bytes, natural alignment) equal offsetof/sizeof of the C structs as
  compiled by gcc from the header, and those of the ctypes mirror used by the tests.
"""
import ctypes
import os
import re
import shutil
import subprocess
import tempfile

import pytest

from peps_mg_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "peps_mg.h")
MODULE = os.path.join(ROOT, "fortran", "peps_mg_gpu.f90")

SIZES = {"c_int": 4, "c_float": 4, "c_double": 8, "c_ptr": 8, "c_long_long": 8}


def header_prototypes():
    """{name: parameter count} of the header's entry points."""
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    out = {}
    for m in re.finditer(r"^(?:int|const char \*)\s*(pmg_\w+)\s*\(([^)]*)\)\s*;", txt, re.M):
        params = m.group(2).strip()
        out[m.group(1)] = 0 if params in ("", "void") else len(params.split(","))
    return out


def module_interfaces():
    """{C name: dummy-argument count} of the module's bind(C) interfaces."""
    src = open(MODULE).read()
    src = re.sub(r"&\s*\n\s*", " ", src)              # join continuation lines
    out = {}
    for m in re.finditer(r"function\s+(\w+)\s*\(([^)]*)\)\s*bind\s*\(\s*C\s*,\s*name\s*=\s*\"(\w+)\"\s*\)", src,
                         re.I):
        args = m.group(2).strip()
        out[m.group(3)] = 0 if not args else len(args.split(","))
    return out


def fortran_type_layout(name):
    """[(component, offset)] and size implied by a bind(C) derived type of the module."""
    src = open(MODULE).read()
    m = re.search(r"type\s*,\s*bind\s*\(\s*C\s*\)\s*,\s*public\s*::\s*%s\s*\n(.*?)end type" % name, src, re.S | re.I)
    assert m, name
    comps = []
    for line in m.group(1).splitlines():
        line = line.split("!")[0].strip()
        if not line:
            continue
        tm = re.match(r"(integer|real|type)\s*\(\s*(\w+)\s*\)\s*::\s*(.*)", line, re.I)
        assert tm, line
        kind = tm.group(2).lower()
        for c in tm.group(3).split(","):
            c = c.strip()
            am = re.match(r"(\w+)\s*\(\s*(\d+)\s*\)", c)
            if am:
                comps.append((am.group(1), kind, int(am.group(2))))
            else:
                comps.append((c, kind, 1))
    off, layout, align = 0, [], 1
    for cname, kind, count in comps:
        sz = SIZES[kind]
        align = max(align, sz)
        off = (off + sz - 1) // sz * sz
        layout.append((cname, off))
        off += sz * count
    size = (off + align - 1) // align * align
    return layout, size


def c_layout(struct, members):
    """offsetof of each member and sizeof, from gcc on the header."""
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "probe.c")
        with open(src, "w") as f:
            f.write('#include <stddef.h>\n#include <stdio.h>\n#include "%s"\nint main(void){\n' % HEADER)
            for mbr in members:
                f.write('printf("%%zu\\n", offsetof(%s, %s));\n' % (struct, mbr))
            f.write('printf("%%zu\\n", sizeof(%s));\nreturn 0;}\n' % struct)
        exe = os.path.join(d, "probe")
        subprocess.run([cc, "-O0", "-o", exe, src], check=True)
        vals = [int(v) for v in subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split()]
    return vals[:-1], vals[-1]


def test_module_binds_every_entry_point():
    protos = header_prototypes()
    ifaces = module_interfaces()
    assert len(protos) >= 30
    missing = sorted(set(protos) - set(ifaces))
    extra = sorted(set(ifaces) - set(protos) - {"strlen"})
    assert not missing, "entry points without a bind(C) interface: %s" % missing
    assert not extra, "interfaces of names the header does not declare: %s" % extra
    for name, n in protos.items():
        assert ifaces[name] == n, (name, ifaces[name], n)


@pytest.mark.parametrize("ftype,cstruct,ctype_cls", [("pmg_config_t", "pmg_config_t", _lib.PmgConfig),
                                                     ("pmg_report_t", "pmg_report_t", _lib.PmgReport)])
def test_bind_c_types_match_the_c_structs(ftype, cstruct, ctype_cls):
    layout, size = fortran_type_layout(ftype)
    names = [n for n, _ in layout]
    offs, csize = c_layout(cstruct, names)
    assert [o for _, o in layout] == offs, (layout, offs)
    assert size == csize
    # the ctypes mirror of the tests and the Python host API
    assert [f[0] for f in ctype_cls._fields_] == names
    assert [getattr(ctype_cls, n).offset for n in names] == offs
    assert ctypes.sizeof(ctype_cls) == csize
