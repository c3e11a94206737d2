"""The CPU oracle reproduces the reference's own traces bit for bit.

The fixtures in tests/golden/ were produced by the reference's unmodified C
(tests/golden/make_golden.py); the oracle starts from the same command-line
parameters and must give identical collision sequences, cells, times and
final states.
"""
import numpy as np
import pytest

from conftest import golden, golden_names, parse_args


@pytest.mark.parametrize("name", golden_names())
def test_oracle_matches_reference(oracle, name):
    g = golden(name)
    a = parse_args(g["args"])
    o = oracle.Oracle(N=a["N"], phi=a["phi"], seed=a["seed"], start=oracle.HEX if a["hex"] else oracle.GROW,
                      xs=a["xs"], q=a["q"], tmax=a["tmax"], additive=bool(g["contact"]), aspect=a["aspect"],
                      res=a["res"], Einit=a["Einit"])
    assert o.N == int(g["N"])
    Lx, Ly, nx, ny = o.box()
    assert (Lx, Ly, nx, ny) == (float(g["Lx"]), float(g["Ly"]), int(g["Nxc"]), int(g["Nyc"]))
    s0 = o.state()
    np.testing.assert_array_equal(s0["x"], g["x0"])
    np.testing.assert_array_equal(s0["vy"], g["vy0"])
    tr, n = o.run(len(g["ct"]))
    assert n == len(g["ct"])
    np.testing.assert_array_equal(tr["i"], g["ci"])
    np.testing.assert_array_equal(tr["j"], g["cj"])
    np.testing.assert_array_equal(tr["cell_i"], g["ccell_i"])
    np.testing.assert_array_equal(tr["cell_j"], g["ccell_j"])
    np.testing.assert_array_equal(tr["t"], g["ct"])
    np.testing.assert_array_equal(o.virial(), g["virial"])
    assert o.t == float(g["t_final"])
    c = o.counters()
    assert (c["ncol"], c["ncross"]) == (int(g["ncol"]), int(g["ncross"]))
    o.sync()
    s = o.state()
    np.testing.assert_array_equal(s["x"], g["xf"])
    np.testing.assert_array_equal(s["y"], g["yf"])
    np.testing.assert_array_equal(s["cell"], g["cellf"])
    np.testing.assert_array_equal(s["coll"].astype(np.int64), g["collf"])
    if "vxf" in g:
        np.testing.assert_array_equal(s["vx"], g["vxf"])
        np.testing.assert_array_equal(s["vy"], g["vyf"])
        np.testing.assert_array_equal(s["rad"], g["radf"])


def test_oracle_conserves_energy_and_momentum(oracle):
    o = oracle.Oracle(N=400, phi=0.6, seed=5, start=oracle.HEX)
    E0, px0, py0 = o.physicalq()
    o.run(50000)
    E1, px1, py1 = o.physicalq()
    assert abs(E1 - E0) / E0 < 1e-12
    assert abs(px1) < 1e-9 and abs(py1) < 1e-9


def test_oracle_no_overlaps(oracle):
    o = oracle.Oracle(N=256, phi=0.72, seed=3, start=oracle.HEX)
    o.run(20000)
    o.sync()
    s = o.state()
    Lx, Ly, _, _ = o.box()
    dx = s["x"][:, None] - s["x"][None, :]
    dy = s["y"][:, None] - s["y"][None, :]
    dx -= Lx * np.round(dx / Lx)
    dy -= Ly * np.round(dy / Ly)
    d2 = dx * dx + dy * dy
    np.fill_diagonal(d2, np.inf)
    assert d2.min() > 4 - 1e-8     # EDMD_VERIFY_OVERLAPS tolerance (src/EDMD.c:4646)


def test_oracle_contact_rules(oracle):
    """Equal radii: (r + r)^2 == 4 r r exactly, so additive contact leaves a
    monodisperse run bit-identical; a bidisperse growth start differs."""
    runs = {}
    for add in (False, True):
        o = oracle.Oracle(N=400, phi=0.6, seed=2, start=oracle.HEX, additive=add)
        tr, n = o.run(3000)
        o.sync()
        runs[add] = (tr.copy(), o.state())
    np.testing.assert_array_equal(runs[False][0]["t"], runs[True][0]["t"])
    np.testing.assert_array_equal(runs[False][1]["x"], runs[True][1]["x"])
    grown = []
    for add in (False, True):
        o = oracle.Oracle(N=200, phi=0.5, seed=4, start=oracle.GROW, xs=0.5, q=0.4, additive=add)
        tr, n = o.run(3000)
        grown.append(tr["t"].copy())
    assert not np.array_equal(grown[0], grown[1])


@pytest.mark.parametrize("name", ["abort_hex8", "abort_grow6"])
def test_oracle_reproduces_reference_abort(built, name):
    """Where the reference stops with its overlap abort (exit(3), EDMD.c:2708-2717),
    the oracle does too, naming the same pair (it exits, so it runs as a child)."""
    import os
    import subprocess
    from conftest import ROOT
    g = golden(name)
    exe = os.path.join(ROOT, "oracle", "oracle_trace")
    r = subprocess.run([exe] + str(g["args"]).split(), env=dict(os.environ, MAXCOLL="1000000", TRACE_OUT=os.devnull),
                       capture_output=True, text=True, timeout=60)
    assert r.returncode == 3
    a, b = int(g["pair"][0]), int(g["pair"][1])
    assert f"overlap between {a} and {b}" in r.stderr, r.stderr
