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
