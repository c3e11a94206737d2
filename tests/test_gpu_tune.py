"""The measured choice of engine and launch shape (graphical-edmd_gb300/tune.py).

Every candidate runs the same trajectories, so the tuner only compares
speeds: it must time every candidate on the batch itself and return the
fastest; the candidate engines must agree on the states they reach.
"""
import numpy as np
import pytest

from conftest import load_pkg_module

pytestmark = pytest.mark.gpu


def test_tuner_times_every_candidate_and_takes_the_fastest(edmd):
    tune = load_pkg_module("tune")
    starts = [edmd.hex_start(256 + 64 * (k % 4), 0.5, 70 + k) for k in range(64)]
    systems = [dict(desc=edmd.default_desc(s["N"], s["Lx"], s["Ly"], 0.0, 1e30), vr=None,
                    **{key: s[key] for key in tune.KEYS}) for s in starts]
    r = tune.tune(edmd, systems, coll=500, reps=1)
    names = {"warp/32", "warp/16", "warp/8", "warp/32/smem", "lane"}
    assert set(r["rates"]) == names
    assert all(v > 0 for v in r["rates"].values())
    assert r["rates"][r["choice"]] == max(r["rates"].values())
    # the candidates reach the same states
    out = []
    for engine, lanes, flags in tune.candidates(edmd, 448):
        if lanes is not None:
            edmd.set_warp_group(lanes)
        eng = edmd.Engine(systems, engine=edmd.ENGINE_LANE if engine == "lane" else edmd.ENGINE_WARP)
        eng.advance(max_coll=500, flags=flags)
        eng.sync()
        out.append(eng.states())
        eng.close()
        edmd.set_warp_group(32)
    for o in out[1:]:
        for k in ("x", "y", "vx", "vy"):
            np.testing.assert_array_equal(o[k], out[0][k])
