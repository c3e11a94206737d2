"""The C-ABI library loads and exports every function the public headers declare.

No compute call is made: this runs on machines without a GPU.
"""
import ctypes
import os
import re

from conftest import ROOT


def declared_functions():
    names = []
    for h in ("edmd_gpu.h", "edmd_host.h"):
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"\b(edmd_\w+)\s*\(", src):
            if m.group(1) not in names:
                names.append(m.group(1))
    return names


def test_library_exports_every_declared_symbol(edmd):
    lib = ctypes.CDLL(edmd.LIB_PATH)
    names = declared_functions()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert sorted(names) == sorted(edmd.EXPORTS)


def test_no_device_reported_cleanly(edmd):
    from conftest import has_gpu
    if has_gpu():
        return
    assert edmd.device_info() is None


def test_struct_layouts_match_the_header(edmd, tmp_path):
    """The ctypes mirrors of the public structs have the header's sizes and
    field offsets (compiled with the host C compiler; no GPU needed)."""
    import subprocess
    structs = {"edmd_system_desc": edmd.SystemDesc, "edmd_collision": edmd.Collision,
               "edmd_counters": edmd.Counters}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "edmd_gpu.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append('printf("%s size %%zu\\n", sizeof(%s));' % (cname, cname))
        for f, _ in py._fields_:
            lines.append('printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, f, cname, f))
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), "-o", str(exe), str(src)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = dict((tuple(l.split()[:2]), int(l.split()[2])) for l in out if l)
    for cname, py in structs.items():
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for f, _ in py._fields_:
            assert got[(cname, f)] == getattr(py, f).offset, (cname, f)
    assert edmd.CONTACT_NONADDITIVE == 0 and edmd.CONTACT_ADDITIVE == 1
    hdr = open(os.path.join(ROOT, "include", "edmd_gpu.h")).read()
    assert re.search(r"#define EDMD_CONTACT_NONADDITIVE 0\b", hdr)
    assert re.search(r"#define EDMD_CONTACT_ADDITIVE\s+1\b", hdr)
