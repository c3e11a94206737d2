"""Shared test fixtures.

GPU tests are marked ``@pytest.mark.gpu``; everything else runs on a CPU-only
machine.  The engine package lives in ``graphical-edmd_gb300/`` (not an
importable name), so it is loaded by path.
"""
import importlib.util
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "graphical-edmd_gb300")
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def load_pkg_module(name):
    key = "edmd_gb300_" + name
    if key in sys.modules:
        return sys.modules[key]
    spec = importlib.util.spec_from_file_location(key, os.path.join(PKG, name + ".py"))
    mod = importlib.util.module_from_spec(spec)
    sys.modules[key] = mod
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="session")
def built():
    """Build the engine library and the oracle once per session."""
    b = load_pkg_module("build")
    b.build()
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    return True


@pytest.fixture(scope="session")
def edmd(built):
    return load_pkg_module("edmd")


@pytest.fixture(scope="session")
def oracle(built):
    from oracle import oracle as o
    return o


def golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False))


def golden_names():
    """Trace fixtures (the files_* and load_* fixtures pin output files instead,
    the abort_* fixtures the reference's overlap abort)."""
    return sorted(f[:-4] for f in os.listdir(GOLDEN)
                  if f.endswith(".npz") and not f.startswith(("files_", "load_", "abort_")))


def parse_args(args):
    """Reference CLI string of a fixture -> start parameters."""
    a = str(args).split()
    out = dict(hex="--hex" in a, N=500, phi=0.38, xs=0.3, q=0.4, seed=1, tmax=4000.0, dtime=100.0,
               dtime_thermo=100.0, res=1.0, Einit=1.0, aspect=1.0)
    keys = {"-N": ("N", int), "--phi": ("phi", float), "-x": ("xs", float), "-q": ("q", float),
            "-v": ("seed", int), "-t": ("tmax", float), "-D": ("dtime", float), "-o": ("dtime_thermo", float),
            "-r": ("res", float), "-E": ("Einit", float), "-a": ("aspect", float)}
    for k, (name, f) in keys.items():
        if k in a:
            out[name] = f(a[a.index(k) + 1])
    return out


def has_gpu():
    try:
        import torch  # noqa: F401
        return torch.cuda.is_available()
    except Exception:
        return False


def line_overlap_state(edmd):
    """59 disks of radius 1 in a 32 x 32 box: a 4-spaced grid with its third
    row taken out, and on that row disk 0 at x = 5, disk 1 at x = 6.5 (0.5
    inside disk 0, moving away from it at speed 1) and disk 2 at x = 8.7
    (moving towards disk 1 at speed 1).  Disks 1 and 2 meet at t = 0.1 and
    swap velocities; disk 1 then approaches disk 0 while still overlapping
    it.  Every other disk drifts at speed ~1e-3."""
    rng = np.random.default_rng(3)
    pts = [(5.0, 10.0), (6.5, 10.0), (8.7, 10.0)]
    for b in range(8):
        if b == 2:
            continue
        for a in range(8):
            pts.append((2.0 + 4 * a, 2.0 + 4 * b))
    N = len(pts)
    x = np.array([p[0] for p in pts])
    y = np.array([p[1] for p in pts])
    vx = rng.uniform(-1e-3, 1e-3, N)
    vy = rng.uniform(-1e-3, 1e-3, N)
    vx[1], vy[1] = 1.0, 0.0
    vx[2], vy[2] = -1.0, 0.0
    desc = edmd.default_desc(N, 32.0, 32.0, 0.0, 1e30)
    return dict(N=N, x=x, y=y, vx=vx, vy=vy, rad=np.ones(N), m=np.ones(N), vr=None, desc=desc)


def names_pair(msg, a, b):
    """True when an engine error message names the overlapping pair (a, b)."""
    return (f"disks {a} and {b}" in msg) or (f"disks {b} and {a}" in msg)
