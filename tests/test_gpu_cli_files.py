"""The drop-in program writes the reference's dump and thermo files byte for byte.

tests/golden/files_*.{dump,thermo} were written by the reference's own
saveTXT / saveThermo (tests/golden/make_golden.py).  The program runs the same
command line on the GPU; since the trajectory is bit-identical, the text
files must be identical too (the hexagonal case: 134,574 collisions, 12
frames, 5 thermo rows).  Each case runs with the serial engine ("warp") and
with the constant-radius phase in rounds ("round"), whose thermo rows are
computed on the host at thermo barriers.
"""
import glob
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, PKG

pytestmark = pytest.mark.gpu


ENGINES = ["warp", "round"]


@pytest.mark.parametrize("engine", ENGINES)
def test_dump_and_thermo_files_identical(built, tmp_path, engine):
    g = dict(np.load(os.path.join(GOLDEN, "files_hex64.npz")))
    args = str(g["args"]).split() + ["--engine", engine]
    exe = os.path.join(PKG, "edmd")
    r = subprocess.run([exe] + args + ["--quiet"], cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r.returncode == 1, r.stderr          # the reference's main returns 1
    dumps = glob.glob(str(tmp_path / "dump" / "*.dump"))
    thermos = glob.glob(str(tmp_path / "dump" / "*.thermo"))
    assert len(dumps) == 1 and len(thermos) == 1
    assert os.path.basename(dumps[0]).startswith("N_64res_1.000phi_0.500000q_0.000rat_0.400Lx_")
    assert open(dumps[0]).read() == open(os.path.join(GOLDEN, "files_hex64.dump")).read()
    assert open(thermos[0]).read() == open(os.path.join(GOLDEN, "files_hex64.thermo")).read()


@pytest.mark.parametrize("engine", ENGINES)
@pytest.mark.parametrize("name", ["load_txt64", "load_dump64"])
def test_restart_files_identical(built, tmp_path, name, engine):
    """-l restarts (src/EDMD.c:980-995, 1366-1451): from a .txt state, with
    velocities drawn from the seed, and from the last frame of a dump, with
    its velocities.  The reference's own run of the same command line wrote
    the golden dump and thermo files (tests/golden/make_golden.py)."""
    g = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    args = str(g["args"]).format(golden=GOLDEN).split() + ["--engine", engine]
    exe = os.path.join(PKG, "edmd")
    r = subprocess.run([exe] + args + ["--quiet"], cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r.returncode == 1, r.stderr
    dumps = glob.glob(str(tmp_path / "dump" / "*.dump"))
    thermos = glob.glob(str(tmp_path / "dump" / "*.thermo"))
    assert len(dumps) == 1 and len(thermos) == 1
    assert open(dumps[0]).read() == open(os.path.join(GOLDEN, name + ".dump")).read()
    assert open(thermos[0]).read() == open(os.path.join(GOLDEN, name + ".thermo")).read()


@pytest.mark.parametrize("engine", ENGINES)
@pytest.mark.parametrize("name", ["files_grow64", "files_add_grow64"])
def test_growth_start_files_identical(built, tmp_path, name, engine):
    """Bidisperse growth start (particlesInit 1690-1829, growth to the
    growth stop, then the constant-radius phase): dump and thermo files as the
    reference writes them, with its default contact rule and with additive
    contact (the reference built with NONADDITIVE 1, src/EDMD.c:35-43; the
    program's --additive)."""
    g = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    args = str(g["args"]).split() + (["--additive"] if int(g["contact"]) else []) + ["--engine", engine]
    exe = os.path.join(PKG, "edmd")
    r = subprocess.run([exe] + args + ["--quiet"], cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r.returncode == 1, r.stderr
    dumps = glob.glob(str(tmp_path / "dump" / "*.dump"))
    thermos = glob.glob(str(tmp_path / "dump" / "*.thermo"))
    assert len(dumps) == 1 and len(thermos) == 1
    assert open(dumps[0]).read() == open(os.path.join(GOLDEN, name + ".dump")).read()
    assert open(thermos[0]).read() == open(os.path.join(GOLDEN, name + ".thermo")).read()


def _run(exe, args, cwd):
    r = subprocess.run([exe] + args + ["--quiet"], cwd=cwd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 1, r.stderr
    (thermo,) = glob.glob(str(cwd / "dump" / "*.thermo"))
    return open(thermo).read().splitlines()


def test_more_thermo_rows_than_the_row_buffer(built, tmp_path):
    """1334 thermo rows in one run (the engine keeps 1024 per system between
    drains): every row is written, in order, and the serial and round-mode
    runs agree on every row's time, collision count and energy."""
    exe = os.path.join(PKG, "edmd")
    args = "--hex -N 64 --phi 0.5 -x 0 -v 9 -t 1200 -D 1000 -o 0.15".split()
    out = {}
    for engine in ENGINES:
        d = tmp_path / engine
        d.mkdir()
        out[engine] = _run(exe, args + ["--engine", engine], d)
    rows = out["warp"][1:]
    t = np.array([float(r.split()[0]) for r in rows])
    assert len(rows) == 1334 and t[0] == 1000.0 and np.all(np.diff(t) > 0)
    assert len(out["round"]) == len(out["warp"])
    for a, b in zip(out["warp"][1:], out["round"][1:]):
        assert a.split()[:3] == b.split()[:3]
