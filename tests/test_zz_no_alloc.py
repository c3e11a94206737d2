"""The allocation-free entry point agrees with the regular one.

edmd_run_noalloc is for callers that cannot allocate device memory (a loop
where cudaMalloc is forbidden, or a host framework that owns every device
buffer): they hand in their own device arrays and the engine keeps all its
working state in one static device array.  This test runs it twice in a row
on device buffers, each time from the same state as the regular path
(edmd_create + edmd_advance + edmd_sync), and requires the same positions,
velocities, collision count and final time -- exactly, as the other parity
tests do.  The file is named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KEYS = ("x", "y", "vx", "vy", "rad", "m")


def test_noalloc_matches_regular_entry_point_twice(edmd):
    import torch
    L = edmd.load()
    s = edmd.hex_start(1024, 0.60, 5)
    desc = edmd.default_desc(s["N"], s["Lx"], s["Ly"])
    dev = torch.device("cuda:0")
    bufs = {k: torch.tensor(s[k], dtype=torch.float64, device=dev) for k in KEYS}
    torch.cuda.synchronize()
    state = {k: s[k].copy() for k in KEYS}
    for call in range(2):
        # regular entry point from the same host state
        eng = edmd.Engine([dict(desc=desc, vr=None, **state)])
        eng.advance(max_coll=3000)
        eng.sync()
        ref = eng.state(0)
        cnt = eng.counters(0)
        eng.close()
        # allocation-free entry point on the caller's device buffers
        ncol, tout = C.c_int64(), C.c_double()
        rc = L.edmd_run_noalloc(C.byref(desc), *[C.c_void_p(bufs[k].data_ptr()) for k in KEYS],
                                3000, float("inf"), C.byref(ncol), C.byref(tout), None)
        assert rc == edmd.OK, L.edmd_last_error(None)
        out = {k: bufs[k].cpu().numpy() for k in KEYS}
        for k in ("x", "y", "vx", "vy"):
            np.testing.assert_array_equal(out[k], ref[k], err_msg=f"call {call}: {k}")
        assert ncol.value == cnt["ncol"] == 3000
        assert tout.value == cnt["t"]
        state = {k: out[k].copy() for k in KEYS}


def test_noalloc_rejects_oversized_systems(edmd):
    L = edmd.load()
    s = edmd.hex_start(10000, 0.70, 1)
    desc = edmd.default_desc(s["N"], s["Lx"], s["Ly"])
    dummy = C.c_void_p(8)   # never dereferenced: the size check comes first
    rc = L.edmd_run_noalloc(C.byref(desc), *([dummy] * 6), 10, float("inf"), None, None, None)
    assert rc == edmd.ERR_CAPACITY
    assert b"8192" in L.edmd_last_error(None)


def _noalloc(L, desc, bufs, max_coll):
    ncol, tout = C.c_int64(), C.c_double()
    rc = L.edmd_run_noalloc(C.byref(desc), *[C.c_void_p(bufs[k].data_ptr()) for k in KEYS],
                            max_coll, float("inf"), C.byref(ncol), C.byref(tout), None)
    return rc, ncol.value, tout.value


def test_noalloc_rejects_positions_outside_the_box_then_runs_again(edmd):
    import torch
    L = edmd.load()
    s = edmd.hex_start(1024, 0.60, 5)
    desc = edmd.default_desc(s["N"], s["Lx"], s["Ly"])
    dev = torch.device("cuda:0")
    bad = {k: s[k].copy() for k in KEYS}
    bad["x"][7] = s["Lx"] + 0.5
    bufs = {k: torch.tensor(bad[k], dtype=torch.float64, device=dev) for k in KEYS}
    rc, ncol, _ = _noalloc(L, desc, bufs, 500)
    assert rc == edmd.ERR_ARG
    assert b"disk 7 outside the box" in L.edmd_last_error(None)
    assert ncol == 0
    # the shared scratch keeps nothing of the failed call
    bufs = {k: torch.tensor(s[k], dtype=torch.float64, device=dev) for k in KEYS}
    rc, ncol, _ = _noalloc(L, desc, bufs, 500)
    assert rc == edmd.OK and ncol == 500


def test_noalloc_reports_an_overlap_met_during_the_run(edmd):
    import torch
    from conftest import line_overlap_state, names_pair
    L = edmd.load()
    s = line_overlap_state(edmd)
    bufs = {k: torch.tensor(s[k], dtype=torch.float64, device="cuda:0") for k in KEYS}
    rc, ncol, tout = _noalloc(L, s["desc"], bufs, 100)
    msg = L.edmd_last_error(None).decode()
    assert rc == edmd.ERR_OVERLAP, msg
    assert names_pair(msg, 0, 1), msg
    assert ncol == 1 and abs(tout - 0.1) < 1e-12


def test_noalloc_additive_contact_matches_oracle(edmd, oracle):
    """A bidisperse packing grown with additive contact (r1 + r2) continues
    in the allocation-free entry point exactly as in the oracle."""
    import torch
    L = edmd.load()
    g = oracle.Oracle(N=300, phi=0.6, seed=8, start=oracle.GROW, xs=0.5, q=0.4, additive=True)
    g.run_growth()
    g.sync()
    st = g.state()
    Lx, Ly, _, _ = g.box()
    start = {k: np.ascontiguousarray(st[k]) for k in KEYS}
    assert set(np.round(start["rad"], 6)) == {0.4, 1.0}
    o = oracle.Oracle(arrays=dict(start, type=st["type"]), Lx=Lx, Ly=Ly, additive=True)
    o.run(2000, cap=1)
    o.sync()
    desc = edmd.default_desc(300, Lx, Ly, contact=edmd.CONTACT_ADDITIVE)
    dev = torch.device("cuda:0")
    bufs = {k: torch.tensor(start[k], dtype=torch.float64, device=dev) for k in KEYS}
    torch.cuda.synchronize()
    ncol, tout = C.c_int64(), C.c_double()
    rc = L.edmd_run_noalloc(C.byref(desc), *[C.c_void_p(bufs[k].data_ptr()) for k in KEYS],
                            2000, float("inf"), C.byref(ncol), C.byref(tout), None)
    assert rc == edmd.OK, L.edmd_last_error(None)
    out = {k: bufs[k].cpu().numpy() for k in KEYS}
    ost = o.state()
    for k in ("x", "y", "vx", "vy"):
        np.testing.assert_array_equal(out[k], ost[k])
    assert ncol.value == 2000 and tout.value == o.t
