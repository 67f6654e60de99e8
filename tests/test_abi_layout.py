"""The ctypes mirrors of the C-ABI descriptors match include/geofd.h: a
probe compiled against the header prints every field's offset and each
struct's size, and the Python structures must agree field by field (a
mismatch would pass wrong arguments silently)."""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "geofd.h")

PAIRS = [("geo_fd2d_desc", "FD2DDesc"), ("geo_fd3d_desc", "FD3DDesc"), ("geo_rtm3d_desc", "RTM3DDesc"),
         ("geo_rtm2d_desc", "RTM2DDesc"), ("geo_rtm2d_gpu_desc", "RTM2DGpuDesc")]


def c_fields(src, name):
    """Field names of `typedef struct name { ... } name;` in declaration order."""
    m = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), src, re.S)
    assert m, name
    body = re.sub(r"/\*.*?\*/", "", m.group(1), flags=re.S)
    names = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        # "const float *theta, *phi" -> theta, phi; "int nx, nz" -> nx, nz
        first, *rest = [p.strip() for p in decl.split(",")]
        names.append(re.findall(r"[A-Za-z_][A-Za-z0-9_]*", first)[-1])
        names += [re.findall(r"[A-Za-z_][A-Za-z0-9_]*", r)[-1] for r in rest]
    return names


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs gcc")
def test_descriptor_layouts_match_header(tmp_path):
    import ctypes as C

    import geophysics_gb300._lib as L
    src = open(HEADER).read()
    probe = ["#include <stdio.h>", "#include <stddef.h>", '#include "geofd.h"', "int main(void) {"]
    for cname, _ in PAIRS:
        probe.append('printf("%s size %%zu\\n", sizeof(%s));' % (cname, cname))
        for f in c_fields(src, cname):
            probe.append('printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, f, cname, f))
    probe.append("return 0; }")
    c_file, exe = tmp_path / "probe.c", tmp_path / "probe"
    c_file.write_text("\n".join(probe))
    subprocess.run(["gcc", "-I" + os.path.dirname(HEADER), str(c_file), "-o", str(exe)], check=True)
    lines = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {}
    for ln in lines:
        if ln:
            s, f, v = ln.split()
            got[(s, f)] = int(v)
    for cname, pyname in PAIRS:
        py = getattr(L, pyname)
        cf = c_fields(src, cname)
        pf = [f[0] for f in py._fields_]
        assert len(cf) == len(pf), (cname, cf, pf)
        for c_name, p_name in zip(cf, pf):
            assert got[(cname, c_name)] == getattr(py, p_name).offset, (cname, c_name, p_name)
        assert got[(cname, "size")] == C.sizeof(py), cname
