"""Failure injection on the host side: every engine turns a bad state or an
exhausted budget into a status code instead of the reference's exit(3).

The reference aborts when a predicted pair overlaps by more than 0.01
(collisionTimeNormal, src/EDMD.c:2708-2717).  Here the faults are made in
host-prepared state -- no GPU is faulted, trapped or hung:

* an overlapping pair in the initial state (caught by the initial
  predictions of edmd_create);
* an overlapping pair that is separating at t = 0, so the initial predictions
  pass it, and becomes approaching after a collision with a third disk at
  t = 0.1: the re-prediction after that collision must report it, in the
  warp, lane and round engines;
* event and round budgets of one (max_events = 1, max_rounds = 1).
"""
import numpy as np
import pytest

from conftest import line_overlap_state, names_pair

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("engine", ["warp", "lane"])
def test_initial_overlap_is_reported_with_its_pair(edmd, engine):
    s = edmd.hex_start(1024, 0.30, 4)
    s["desc"] = edmd.default_desc(s["N"], s["Lx"], s["Ly"])
    # move disk 600 to 1.5 from disk 0 (between two lattice neighbours of
    # disk 0), the pair approaching: an overlap of 0.5 in a distance of 2
    ang = np.pi / 6
    s["x"][600] = (s["x"][0] + 1.5 * np.cos(ang)) % s["Lx"]
    s["y"][600] = (s["y"][0] + 1.5 * np.sin(ang)) % s["Ly"]
    s["vx"][0], s["vy"][0] = np.cos(ang), np.sin(ang)
    s["vx"][600], s["vy"][600] = -np.cos(ang), -np.sin(ang)
    with pytest.raises(edmd.EngineError) as ei:
        edmd.Engine([s], engine=edmd.ENGINE_LANE if engine == "lane" else edmd.ENGINE_WARP)
    assert ei.value.code == edmd.ERR_OVERLAP
    assert names_pair(str(ei.value), 0, 600), str(ei.value)


@pytest.mark.parametrize("engine", ["warp", "lane", "round"])
def test_overlap_met_during_the_run_is_reported(edmd, engine):
    s = line_overlap_state(edmd)
    eng = edmd.Engine([s], engine=edmd.ENGINE_LANE if engine == "lane" else edmd.ENGINE_WARP)
    if engine == "round":
        rc = eng.advance_rounds(max_coll=100, radius=3, check=False)[0]
    else:
        rc = eng.advance(max_coll=100, check=False)[0]
    msg = eng.last_error()
    assert rc == edmd.ERR_OVERLAP, msg
    assert names_pair(msg, 0, 1), msg
    if engine != "round":
        c = eng.counters(0)
        assert c["ncol"] == 1 and abs(c["t"] - 0.1) < 1e-12     # stopped at the 1-2 collision
    eng.close()


@pytest.mark.parametrize("engine", ["warp", "lane"])
def test_event_budget_of_one(edmd, engine):
    s = edmd.hex_start(1024, 0.60, 2)
    s["desc"] = edmd.default_desc(s["N"], s["Lx"], s["Ly"])
    eng = edmd.Engine([s], engine=edmd.ENGINE_LANE if engine == "lane" else edmd.ENGINE_WARP)
    rc = eng.advance(max_coll=1000, max_events=1, check=False)[0]
    assert rc == edmd.ERR_BUDGET
    assert "event budget" in eng.last_error()
    assert eng.counters(0)["nevents"] == 1
    eng.close()


def test_round_budget_of_one(edmd):
    s = edmd.hex_start(20000, 0.70, 2)
    s["desc"] = edmd.default_desc(s["N"], s["Lx"], s["Ly"])
    eng = edmd.Engine([s])
    rc, _, rounds, _ = eng.advance_rounds(max_coll=10 ** 6, radius=3, max_rounds=1, check=False)
    assert rc == edmd.ERR_BUDGET
    assert "round budget" in eng.last_error()
    # rounds run in graph-captured groups: the budget stops at the first group
    assert rounds >= 1 and 0 < eng.counters(0)["ncol"] < 10 ** 6
    eng.close()


@pytest.mark.parametrize("bad", [-1.0, 1e-310, float("nan"), float("inf")])
def test_invalid_radius_is_an_argument_error(edmd, bad):
    """Radii must be zero or normal positive: the contact distance takes 4 r
    exactly on the integer pipe, which holds for those."""
    s = edmd.hex_start(256, 0.30, 4)
    s["desc"] = edmd.default_desc(s["N"], s["Lx"], s["Ly"])
    s["rad"] = s["rad"].copy()
    s["rad"][17] = bad
    with pytest.raises(edmd.EngineError) as ei:
        edmd.Engine([s])
    assert ei.value.code == edmd.ERR_ARG
    assert "radius" in str(ei.value)


@pytest.mark.parametrize("engine", ["warp", "lane", "round"])
@pytest.mark.parametrize("name", ["abort_hex8", "abort_grow6"])
def test_reference_abort_reproduced(edmd, name, engine):
    """Boxes of three cells a side where the reference itself stops with its
    overlap abort (collisionTimeNormal, src/EDMD.c:2708-2717, exit(3)) after a
    few dozen collisions (tests/golden/make_golden.py).  The engine accepts
    the same collisions, in the same order at the same times, and then
    reports EDMD_ERR_OVERLAP naming the pair the reference names.  The round
    engine runs the constant-radius phase only, so it takes the Hex case, and
    is held to the status and the pair."""
    from conftest import golden, parse_args
    g = golden(name)
    a = parse_args(g["args"])
    if engine == "round" and not a["hex"]:
        pytest.skip("the round engine runs the constant-radius phase only")
    N = int(g["N"])
    if a["hex"]:
        vr, vr_base = None, 0.0
    else:
        st = edmd.grow_start(a["N"], a["phi"], a["seed"], xs=a["xs"], q=a["q"])
        vr, vr_base = st["vr"], st["vr_base"]
    desc = edmd.default_desc(N, float(g["Lx"]), float(g["Ly"]), vr_base, a["tmax"], a["dtime"], a["dtime_thermo"])
    s = dict(desc=desc, x=g["x0"], y=g["y0"], vx=g["vx0"], vy=g["vy0"], rad=g["rad0"], m=g["m0"], vr=vr)
    n = len(g["ct"])
    eng = edmd.Engine([s], trace_cap=n + 16, engine=edmd.ENGINE_LANE if engine == "lane" else edmd.ENGINE_WARP)
    if engine == "round":
        rc = eng.advance_rounds(max_coll=10 ** 6, radius=3, flags=edmd.F_TRACE, check=False)[0]
    else:
        rc = eng.advance(max_coll=10 ** 6, flags=edmd.F_TRACE, check=False)[0]
    msg = eng.last_error()
    assert rc == edmd.ERR_OVERLAP, msg
    assert names_pair(msg, int(g["pair"][0]), int(g["pair"][1])), msg
    if engine != "round":
        # (a round also runs the events selected beside the failing one)
        tr = eng.trace(0)
        assert len(tr) == n
        np.testing.assert_array_equal(tr["i"], g["ci"])
        np.testing.assert_array_equal(tr["j"], g["cj"])
        np.testing.assert_array_equal(tr["t"], g["ct"])
    eng.close()
