"""Device g(r) (calculate_pcf, src/pcf.c:16-75) against the oracle, bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("N,phi,coll,max_r", [(2000, 0.70, 20000, None), (20000, 0.72, 50000, 12.0),
                                              (4096, 0.40, 5000, None)])
def test_pcf_matches_oracle(edmd, oracle, N, phi, coll, max_r):
    s = edmd.hex_start(N, phi, 5)
    eng = edmd.Engine([dict(desc=edmd.default_desc(s["N"], s["Lx"], s["Ly"]), **s)])
    eng.advance(max_coll=coll)
    eng.sync()
    o = oracle.Oracle(arrays={k: s[k] for k in ("x", "y", "vx", "vy", "rad", "m", "type")}, Lx=s["Lx"], Ly=s["Ly"])
    o.run(coll, cap=1)
    o.sync()
    mr = max_r if max_r is not None else min(s["Lx"], s["Ly"]) / 2
    r, g = eng.pcf(0, 0.1, mr)
    ro, go = o.pcf(0.1, mr)
    assert len(g) == len(go) == int(mr / 0.1)
    np.testing.assert_array_equal(r, ro)
    np.testing.assert_array_equal(g, go)
    # a dense liquid: first peak near contact (diameter 2), g -> 1 far away
    assert g[int(2.0 / 0.1)] > 1.5 and abs(g[-20:].mean() - 1) < 0.1
