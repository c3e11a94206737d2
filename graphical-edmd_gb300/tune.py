"""Measured choice of engine and launch shape for a batch of systems.

Every engine and launch shape of the serial-exact event loop gives
bit-identical trajectories (the reference's event order), so the choice is a
pure speed question, and the answer depends on the batch: the warp engine
(one system per 32-lane group) wins for a few thousand systems, narrower
groups trade FP64 issue against divergence, the shared-memory kernel trades
memory latency against resident systems, and the thread-per-system engine
wins once there are tens of thousands of systems.  `tune` times each
candidate on the batch itself -- a fresh context from the given states, one
untimed warm-up call and `reps` timed calls of `coll` accepted collisions per
system (CUDA events on the context's stream) -- and returns the fastest.

Candidates: (engine, lanes per system, advance flags); lanes is None for the
thread-per-system engine.
"""
import numpy as np

KEYS = ("x", "y", "vx", "vy", "rad", "m")


def candidates(edmd, max_n):
    out = [("warp", 32, 0), ("warp", 16, 0), ("warp", 8, 0), ("warp", 32, edmd.F_SMEM)]
    if 2 * max_n + 3 <= 65535:
        out.append(("lane", None, 0))
    return out


def _rate(edmd, systems, engine, lanes, flags, coll, reps):
    if lanes is not None:
        edmd.set_warp_group(lanes)
    eng = edmd.Engine(systems, engine=edmd.ENGINE_LANE if engine == "lane" else edmd.ENGINE_WARP)
    try:
        eng.advance(max_coll=coll, flags=edmd.F_COUNT_NORMAL | flags)
        c0 = eng.all_counters()["ncol"].sum()
        ms = 0.0
        for _ in range(reps):
            ms += eng.advance(max_coll=coll, flags=edmd.F_COUNT_NORMAL | flags)[1]
        n = eng.all_counters()["ncol"].sum() - c0
    finally:
        eng.close()
        edmd.set_warp_group(32)
    return float(n) / (ms / 1000.0)


def tune(edmd, systems, coll=2000, reps=2):
    """systems: dicts with desc, x, y, vx, vy, rad, m (normal phase).  Returns
    {"engine", "lanes", "flags", "rates": {name: coll/s}}."""
    max_n = max(s["desc"].N for s in systems)
    rates = {}
    best = None
    for engine, lanes, flags in candidates(edmd, max_n):
        name = engine + ("" if lanes is None else "/%d" % lanes) + ("/smem" if flags else "")
        r = _rate(edmd, systems, engine, lanes, flags, coll, reps)
        rates[name] = r
        if best is None or r > best[0]:
            best = (r, engine, lanes, flags, name)
    return {"engine": best[1], "lanes": best[2], "flags": best[3], "choice": best[4], "rates": rates}


def systems_from_states(desc, states, N):
    """Per-system dicts from concatenated states (edmd.Engine.states())."""
    off = np.cumsum([0] + list(N))
    out = []
    for k, d in enumerate(desc):
        sl = slice(off[k], off[k + 1])
        out.append(dict(desc=d, vr=None, **{key: np.ascontiguousarray(states[key][sl]) for key in KEYS}))
    return out
