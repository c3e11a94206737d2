"""Round-parallel engine == reference, through the C ABI.

The round engine processes many causally independent events at once, so the
order of its trace differs from the reference's; everything else is checked
exactly: the set of accepted collisions (unordered pair, contact time and the
pair's cells), the collision and crossing counters, the final positions,
velocities, cells and collision counters.  The virial sums differ only by the
order of the floating-point additions (relative 1e-12).  Runs use
EDMD_F_EXACT, which replays a call from its start with a wider window whenever
a causality violation was detected, so the comparison holds whatever the
violation count.
"""
import numpy as np
import pytest

from conftest import golden, golden_names, parse_args

pytestmark = pytest.mark.gpu

HEX = [n for n in golden_names() if n.startswith("hex") or (n.startswith(("opt_", "tiny_")) and n.endswith(("_hex", "hex12")))]


def canon(i, j, ci, cj, t):
    """Collision records as a sorted array of (t, lo, hi, cell_lo, cell_hi)."""
    lo, hi = np.minimum(i, j), np.maximum(i, j)
    clo = np.where(i <= j, ci, cj)
    chi = np.where(i <= j, cj, ci)
    rec = np.zeros(len(t), [("t", "<f8"), ("lo", "<i8"), ("hi", "<i8"), ("clo", "<i8"), ("chi", "<i8")])
    rec["t"], rec["lo"], rec["hi"], rec["clo"], rec["chi"] = t, lo, hi, clo, chi
    return np.sort(rec, order=("t", "lo", "hi"))


def system_from_golden(edmd, g):
    a = parse_args(g["args"])
    desc = edmd.default_desc(int(g["N"]), float(g["Lx"]), float(g["Ly"]))
    desc.res, desc.Einit = a["res"], a["Einit"]
    return dict(desc=desc, x=g["x0"], y=g["y0"], vx=g["vx0"], vy=g["vy0"], rad=g["rad0"], m=g["m0"])


def check_golden(edmd, eng, s, g):
    tr = eng.trace(s)
    n = len(g["ct"])
    assert len(tr) == n
    a = canon(tr["i"], tr["j"], tr["cell_i"], tr["cell_j"], tr["t"])
    b = canon(g["ci"], g["cj"], g["ccell_i"], g["ccell_j"], g["ct"])
    assert a.tobytes() == b.tobytes()
    c = eng.counters(s)
    assert c["t"] == float(g["t_final"])
    assert (c["ncol"], c["ncross"]) == (int(g["ncol"]), int(g["ncross"]))
    np.testing.assert_allclose(eng.virial(s), g["virial"], rtol=1e-12, atol=1e-12 * np.abs(g["virial"]).max())
    st = eng.state(s)
    np.testing.assert_array_equal(st["x"], g["xf"])
    np.testing.assert_array_equal(st["y"], g["yf"])
    np.testing.assert_array_equal(st["cell"], g["cellf"])
    np.testing.assert_array_equal(st["coll"].astype(np.int64), g["collf"])


EXACT = 32   # EDMD_F_EXACT (include/edmd_gpu.h)


@pytest.mark.parametrize("radius", [3, 5])
@pytest.mark.parametrize("name", HEX)
def test_rounds_match_reference_collisions(edmd, name, radius):
    g = golden(name)
    eng = edmd.Engine([system_from_golden(edmd, g)], trace_cap=len(g["ct"]) + 16)
    t_stop = np.nextafter(float(g["t_final"]), np.inf)
    rc, ms, rounds, viol = eng.advance_rounds(t_stop=t_stop, flags=edmd.F_TRACE | EXACT, radius=radius)
    eng.sync()
    check_golden(edmd, eng, 0, g)
    eng.close()


def oracle_run_to(oracle, start, t_stop):
    o = oracle.Oracle(arrays={k: start[k] for k in ("x", "y", "vx", "vy", "rad", "m", "type")},
                      Lx=start["Lx"], Ly=start["Ly"])
    _, n = o.run(10 ** 12, t_stop=t_stop, cap=1)
    o.sync()
    return o, n


@pytest.mark.parametrize("N,phi,seed,t_stop,mode", [(20000, 0.72, 5, 3.0, 0), (4096, 0.45, 6, 12.0, 0),
                                                     (100000, 0.72, 8, 0.6, 0), (100000, 0.72, 8, 0.6, 1),
                                                     (640000, 0.72, 9, 0.25, 1), (640000, 0.72, 9, 0.25, 2),
                                                     (640000, 0.72, 9, 0.5, 0)])
def test_rounds_match_oracle_state(edmd, oracle, N, phi, seed, t_stop, mode):
    """Larger systems against the oracle: counters, final state, screenshot at t = 1.
    mode 1 runs every round one thread per event, mode 2 adds the FP32 screen
    of separating pairs.  The 640,000-disk system in mode 0 has rounds of more
    events than k_process has resident warps, so warps past their first event
    take the rest of a round from its counter."""
    s = edmd.hex_start(N, phi, seed)
    o, n = oracle_run_to(oracle, s, t_stop)
    eng = edmd.Engine([dict(desc=edmd.default_desc(s["N"], s["Lx"], s["Ly"]), **s)])
    fl = EXACT | (edmd.F_ROUND_THREAD if mode else 0) | (edmd.F_SCREEN if mode == 2 else 0)
    rc, ms, rounds, viol = eng.advance_rounds(t_stop=t_stop, radius=3, flags=fl)
    eng.sync()
    c = eng.counters(0)
    oc = o.counters()
    assert (c["ncol"], c["ncross"]) == (oc["ncol"], oc["ncross"]) and c["ncol"] == n
    assert c["t"] == o.t
    assert (c["nscreen"] > 0) == (mode == 2)
    if mode == 0 and N >= 640000:
        torch = pytest.importorskip("torch")
        wave = 20 * torch.cuda.get_device_properties(0).multi_processor_count   # one-warp blocks, 20 per SM
        assert c["nevents"] / rounds > wave      # rounds counts whole 32-round graphs: an underestimate
    st, ost = eng.state(0), o.state()
    for k in ("x", "y", "vx", "vy"):
        np.testing.assert_array_equal(st[k], ost[k])
    np.testing.assert_array_equal(st["cell"], ost["cell"])
    np.testing.assert_array_equal(st["coll"].astype(np.uint64), ost["coll"])
    np.testing.assert_allclose(eng.virial(0), o.virial(), rtol=1e-11)
    eng.close()


def test_rounds_batch_matches_oracle(edmd, oracle):
    """Systems of uneven N and density in one context, each against the oracle."""
    cases = [(256, 0.30, 11), (1000, 0.70, 12), (2000, 0.55, 13), (4096, 0.74, 14), (700, 0.62, 15)]
    starts = [edmd.hex_start(N, phi, seed) for N, phi, seed in cases]
    t_stop = 4.0
    eng = edmd.Engine([dict(desc=edmd.default_desc(s["N"], s["Lx"], s["Ly"]), **s) for s in starts])
    rc, ms, rounds, viol = eng.advance_rounds(t_stop=t_stop, radius=3, flags=EXACT)
    eng.sync()
    for k, s in enumerate(starts):
        o, n = oracle_run_to(oracle, s, t_stop)
        st, ost = eng.state(k), o.state()
        for key in ("x", "y", "vx", "vy"):
            np.testing.assert_array_equal(st[key], ost[key])
        c, oc = eng.counters(k), o.counters()
        assert (c["ncol"], c["ncross"]) == (oc["ncol"], oc["ncross"])
        assert c["t"] == o.t
    eng.close()


@pytest.mark.parametrize("contact", ["default", "additive", "mixed"])
def test_rounds_bidisperse_batch_after_growth(edmd, oracle, contact):
    """Growth on the serial engine, then the constant-radius phase in rounds;
    with the reference's contact rule, additive contact (r1 + r2), or the two
    mixed in one batch."""
    starts = [edmd.grow_start(n, phi, seed, xs=0.5, q=0.7142857)
              for n, phi, seed in ((400, 0.70, 3), (1000, 0.55, 4), (256, 0.35, 5))]
    add = [{"default": 0, "additive": 1, "mixed": k % 2}[contact] for k in range(len(starts))]
    systems = []
    for k, s in enumerate(starts):
        d = edmd.default_desc(s["N"], s["Lx"], s["Ly"], s["vr_base"], contact=add[k])
        systems.append(dict(desc=d, **{k: s[k] for k in ("x", "y", "vx", "vy", "rad", "m", "vr")}))
    eng = edmd.Engine(systems)
    eng.advance(flags=edmd.F_STOP_AT_GROW)
    t_stop = max(1 / s["vr_base"] for s in starts) + 5.0
    rc, ms, rounds, viol = eng.advance_rounds(t_stop=t_stop, radius=3, flags=EXACT)
    eng.sync()
    for k, s in enumerate(starts):
        o = oracle.Oracle(N=s["N"], phi=[0.70, 0.55, 0.35][k], seed=[3, 4, 5][k], start=oracle.GROW,
                          xs=0.5, q=0.7142857, additive=bool(add[k]))
        o.run(10 ** 12, t_stop=t_stop, cap=1)
        o.sync()
        st, ost = eng.state(k), o.state()
        for key in ("x", "y", "vx", "vy", "rad"):
            np.testing.assert_array_equal(st[key], ost[key])
        c, oc = eng.counters(k), o.counters()
        assert (c["ncol"], c["ncross"]) == (oc["ncol"], oc["ncross"])
    eng.close()


def test_serial_engine_refuses_after_rounds(edmd):
    s = edmd.hex_start(1024, 0.6, 1)
    eng = edmd.Engine([dict(desc=edmd.default_desc(s["N"], s["Lx"], s["Ly"]), **s)])
    eng.advance_rounds(t_stop=0.5, flags=EXACT)
    rc, _ = eng.advance(max_coll=10, check=False)
    assert rc == edmd.ERR_ARG
    eng.sync()
    st = eng.state(0)
    eng.load_state(st["x"], st["y"], st["vx"], st["vy"], st["rad"], st["m"])
    rc, _ = eng.advance(max_coll=10, check=False)
    assert rc == edmd.OK
    eng.close()


def test_collision_budget_ends_on_a_serial_state(edmd, oracle):
    """A stop at max_coll drains the earlier pending events: the state is the
    oracle's at the same time, and a second call continues it exactly."""
    s = edmd.hex_start(20000, 0.70, 21)
    eng = edmd.Engine([dict(desc=edmd.default_desc(s["N"], s["Lx"], s["Ly"]), **s)])
    for _ in range(2):
        eng.advance_rounds(max_coll=30000, radius=3, flags=EXACT)
        c = eng.counters(0)
        assert c["stop_reason"] == edmd.STOP_COLL and c["ncol"] >= 30000
    eng.sync()
    o, n = oracle_run_to(oracle, s, np.nextafter(c["t"], np.inf))
    assert n == c["ncol"] and o.t == c["t"]
    st, ost = eng.state(0), o.state()
    for k in ("x", "y", "vx", "vy"):
        np.testing.assert_array_equal(st[k], ost[k])
    eng.close()


def test_exact_mode_replays_to_the_same_result(edmd):
    """The window radius changes the rounds, never the result."""
    s = edmd.hex_start(50000, 0.72, 22)
    out = []
    for radius in (3, 6):
        eng = edmd.Engine([dict(desc=edmd.default_desc(s["N"], s["Lx"], s["Ly"]), **s)])
        eng.advance_rounds(t_stop=1.5, radius=radius, flags=EXACT)
        eng.sync()
        out.append((eng.state(0), eng.counters(0)))
        eng.close()
    for k in ("x", "y", "vx", "vy", "coll"):
        np.testing.assert_array_equal(out[0][0][k], out[1][0][k])
    assert out[0][1]["ncol"] == out[1][1]["ncol"]


def test_block_rounds_match_grid_rounds_and_oracle(edmd, oracle):
    """One block per system gives the grid-wide engine's result, and the oracle's."""
    rng = np.random.default_rng(31)
    cases = [(int(n), float(p), 100 + k) for k, (n, p) in
             enumerate(zip(rng.integers(256, 1500, 160), rng.uniform(0.3, 0.72, 160)))]
    starts = [edmd.hex_start(N, phi, seed) for N, phi, seed in cases]
    systems = [dict(desc=edmd.default_desc(s["N"], s["Lx"], s["Ly"]), **s) for s in starts]
    t_stop = 1.5
    out = []
    for mode in (edmd.F_ROUND_BLOCK, edmd.F_ROUND_GRID):
        eng = edmd.Engine(systems)
        rc, ms, rounds, viol = eng.advance_rounds(t_stop=t_stop, radius=3, flags=EXACT | mode)
        eng.sync()
        out.append(eng.states())
        cb = eng.all_counters()
        eng.close()
    for k in ("x", "y", "vx", "vy"):
        np.testing.assert_array_equal(out[0][k], out[1][k])
    off = np.cumsum([0] + [s["N"] for s in starts])
    for q in (0, 57, 159):
        o, n = oracle_run_to(oracle, starts[q], t_stop)
        ost = o.state()
        for k in ("x", "y", "vx", "vy"):
            np.testing.assert_array_equal(out[0][k][off[q]:off[q + 1]], ost[k])
        assert cb["ncol"][q] == o.counters()["ncol"]


def test_block_rounds_collision_budget(edmd, oracle):
    """Block mode with a collision budget per system ends on serial states."""
    cases = [(300 + 7 * k, 0.5 + 0.001 * k, 200 + k) for k in range(160)]
    starts = [edmd.hex_start(N, phi, seed) for N, phi, seed in cases]
    eng = edmd.Engine([dict(desc=edmd.default_desc(s["N"], s["Lx"], s["Ly"]), **s) for s in starts])
    eng.advance_rounds(max_coll=2000, radius=3, flags=EXACT | edmd.F_ROUND_BLOCK)
    c = eng.all_counters()
    assert (c["ncol"] >= 2000).all() and (c["stop_reason"] == edmd.STOP_COLL).all()
    eng.sync()
    for q in (3, 99):
        o, n = oracle_run_to(oracle, starts[q], np.nextafter(c["t"][q], np.inf))
        assert n == c["ncol"][q]
        np.testing.assert_array_equal(eng.state(q)["x"], o.state()["x"])
    eng.close()


def test_launch_counts_are_reported(edmd):
    """edmd_get_last_launches: one persistent launch per serial call; per round
    the selection, event and recompute/barrier kernels (and the thread-per-event
    kernel in the graphs that hold it), plus the call's set-up and finish."""
    s = edmd.hex_start(20000, 0.70, 3)
    s["desc"] = edmd.default_desc(s["N"], s["Lx"], s["Ly"])
    eng = edmd.Engine([s])
    eng.advance(max_coll=1000)
    assert eng.last_launches() == 1
    rc, ms, rounds, viol = eng.advance_rounds(max_coll=20000, radius=4, flags=EXACT)
    n = eng.last_launches()
    assert rounds > 0 and 3 * rounds + 4 <= n <= 4 * rounds + 5, (n, rounds)
    eng.close()
