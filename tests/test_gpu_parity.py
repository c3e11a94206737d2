"""GPU engine == reference, bit for bit, through the C ABI.

Each fixture holds the reference's initial state, its first accepted
collisions (owner i, partner j, their cells, time) and the state after the
last one.  The engine starts from the same state and must reproduce the
ordered (i, j) pairs, the cells, the times, the virial sums, the counters and
the final positions/velocities exactly (integer and index results bit-exact;
positions are compared exactly, which is stricter than the 1e-12 bound).
The add_* fixtures come from the reference built with additive contact
(NONADDITIVE 1, src/EDMD.c:35-43) and run with edmd_system_desc.contact =
EDMD_CONTACT_ADDITIVE; batches mix them with the default-contact systems.
"""
import numpy as np
import pytest

from conftest import golden, golden_names, parse_args

pytestmark = pytest.mark.gpu


def system_from_golden(edmd, g):
    a = parse_args(g["args"])
    N = int(g["N"])
    if a["hex"]:
        vr, vr_base = None, 0.0
    else:
        s = edmd.grow_start(a["N"], a["phi"], a["seed"], xs=a["xs"], q=a["q"], aspect=a["aspect"])
        vr, vr_base = s["vr"], s["vr_base"]
    desc = edmd.default_desc(N, float(g["Lx"]), float(g["Ly"]), vr_base, a["tmax"], a["dtime"],
                             a["dtime_thermo"], contact=int(g["contact"]))
    desc.res, desc.Einit = a["res"], a["Einit"]
    return dict(desc=desc, x=g["x0"], y=g["y0"], vx=g["vx0"], vy=g["vy0"], rad=g["rad0"], m=g["m0"], vr=vr)


def check_against_golden(eng, s, g):
    tr = eng.trace(s)
    n = len(g["ct"])
    assert len(tr) == n
    np.testing.assert_array_equal(tr["i"], g["ci"])
    np.testing.assert_array_equal(tr["j"], g["cj"])
    np.testing.assert_array_equal(tr["cell_i"], g["ccell_i"])
    np.testing.assert_array_equal(tr["cell_j"], g["ccell_j"])
    np.testing.assert_array_equal(tr["t"], g["ct"])
    c = eng.counters(s)
    assert c["t"] == float(g["t_final"])
    assert (c["ncol"], c["ncross"]) == (int(g["ncol"]), int(g["ncross"]))
    np.testing.assert_array_equal(eng.virial(s), g["virial"])
    st = eng.state(s)
    np.testing.assert_array_equal(st["x"], g["xf"])
    np.testing.assert_array_equal(st["y"], g["yf"])
    np.testing.assert_array_equal(st["cell"], g["cellf"])
    np.testing.assert_array_equal(st["coll"].astype(np.int64), g["collf"])
    if "vxf" in g:
        np.testing.assert_array_equal(st["vx"], g["vxf"])
        np.testing.assert_array_equal(st["vy"], g["vyf"])
        np.testing.assert_array_equal(st["rad"], g["radf"])


ENGINES = [("warp", 1), ("lane", 2)]


@pytest.mark.parametrize("engine", ENGINES, ids=[e[0] for e in ENGINES])
@pytest.mark.parametrize("name", golden_names())
def test_single_system_matches_reference(edmd, name, engine):
    g = golden(name)
    eng = edmd.Engine([system_from_golden(edmd, g)], trace_cap=len(g["ct"]) + 16, engine=engine[1])
    assert eng.engine == engine[1]
    rc, ms = eng.advance(max_coll=len(g["ct"]), flags=edmd.F_TRACE)
    eng.sync()
    check_against_golden(eng, 0, g)
    eng.close()


@pytest.mark.parametrize("engine", ENGINES, ids=[e[0] for e in ENGINES])
def test_batched_systems_match_reference(edmd, engine):
    """Several systems of different N in one launch, each replicated 3 times."""
    by_len = {}
    for n in golden_names():
        g = golden(n)
        by_len.setdefault(len(g["ct"]), []).append(g)
    for L, gs in sorted(by_len.items()):
        systems = [system_from_golden(edmd, g) for g in gs] * 3
        eng = edmd.Engine(systems, trace_cap=L + 16, engine=engine[1])
        eng.advance(max_coll=L, flags=edmd.F_TRACE)
        eng.sync()
        for s in range(len(systems)):
            check_against_golden(eng, s, gs[s % len(gs)])
        eng.close()


def test_batch_larger_than_resident_warps(edmd, oracle):
    """More systems than resident warps: from the second call on, the systems
    are taken longest-first by their previous run time; every system still
    gives the oracle's result."""
    starts = [edmd.hex_start(256 + 16 * (k % 7), 0.45 + 0.04 * (k % 7), 500 + k) for k in range(2600)]
    eng = edmd.Engine([dict(desc=edmd.default_desc(s["N"], s["Lx"], s["Ly"]), **s) for s in starts])
    for _ in range(3):
        eng.advance(max_coll=1000)
    eng.sync()
    assert (eng.all_counters()["ncol"] == 3000).all()
    for q in (0, 1300, 2599):
        s = starts[q]
        o = oracle.Oracle(arrays={k: s[k] for k in ("x", "y", "vx", "vy", "rad", "m", "type")},
                          Lx=s["Lx"], Ly=s["Ly"])
        o.run(3000, cap=1)
        o.sync()
        st = eng.state(q)
        for k in ("x", "y", "vx", "vy"):
            np.testing.assert_array_equal(st[k], o.state()[k])
    eng.close()


@pytest.mark.parametrize("lanes", [32, 16, 8, 4])
def test_warp_group_widths_match_reference(edmd, lanes):
    """One system per warp (32 lanes) and two, four or eight per warp (16, 8
    or 4 lanes each): the same collisions, cells, times and states as the
    reference."""
    try:
        edmd.set_warp_group(lanes)
        names = golden_names()
        gs = [golden(n) for n in names]
        L = min(len(g["ct"]) for g in gs)
        systems = [system_from_golden(edmd, g) for g in gs] * 5
        eng = edmd.Engine(systems, trace_cap=L + 16)
        for g in gs:
            assert len(g["ct"]) >= L
        eng.advance(max_coll=L, flags=edmd.F_TRACE)
        eng.sync()
        for s, g in enumerate(gs * 5):
            tr = eng.trace(s)
            assert len(tr) == L
            for k, gk in (("i", "ci"), ("j", "cj"), ("cell_i", "ccell_i"), ("cell_j", "ccell_j"), ("t", "ct")):
                np.testing.assert_array_equal(tr[k], g[gk][:L])
        eng.close()
    finally:
        edmd.set_warp_group(32)


def test_shared_memory_kernel_matches_reference(edmd):
    """EDMD_F_SMEM: the systems whose state fits a block's shared memory run
    from there (the 10^4-disk fixture does not fit and runs in the regular
    kernel beside them); every system still reproduces the reference."""
    by_len = {}
    for n in golden_names():
        g = golden(n)
        by_len.setdefault(len(g["ct"]), []).append(g)
    for L, gs in sorted(by_len.items()):
        systems = [system_from_golden(edmd, g) for g in gs] * 3
        eng = edmd.Engine(systems, trace_cap=L + 16)
        eng.advance(max_coll=L, flags=edmd.F_TRACE | edmd.F_SMEM)
        eng.sync()
        for s in range(len(systems)):
            check_against_golden(eng, s, gs[s % len(gs)])
        eng.close()
