"""Tangent-linear and adjoint kernels against FP64 central finite differences.

Finite differences come from the CPU oracle (the reference's serial algorithm),
run from initial states displaced by +-eps (eps = 1e-7) along a direction, to
a fixed observation time t_obs placed between the n-th and (n+1)-th collision
of the unperturbed run (n = 1000 for the adjoint, 300 for the full 4N tangent
direction); each perturbed run must process the same collisions, otherwise the
comparison is meaningless.  The MSD displacement is measured from the
(perturbed) initial positions, so its gradient with respect to r(0) includes
the direct term.  Tolerances: 1e-5 relative (tangent,
full 4N vector) and 1e-6 relative (adjoint gradient components, the north-star
figure), both far above the O(eps^2) truncation and the 1e-9 roundoff of the
differences.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

EPS = 1e-7
NCOLL = 1000


def make_setup(edmd, oracle, ncoll):
    """A generic N = 1024, phi = 0.60 state (the Hex start run 3000 collisions)."""
    s = edmd.hex_start(1024, 0.60, 11)
    o = oracle.Oracle(arrays={k: s[k] for k in ("x", "y", "vx", "vy", "rad", "m", "type")},
                      Lx=s["Lx"], Ly=s["Ly"])
    o.run(3000)
    o.sync()
    st = o.state()
    init = {k: st[k].copy() for k in ("x", "y", "vx", "vy", "rad", "m")}
    init["type"] = st["type"].copy()
    # unperturbed reference run: observation time between collisions ncoll and ncoll+1
    ob = oracle.Oracle(arrays=init, Lx=s["Lx"], Ly=s["Ly"])
    tr, n = ob.run(ncoll + 1)
    T, t_next = tr["t"][ncoll - 1], tr["t"][ncoll]
    assert t_next > T
    t_obs = T + 0.25 * (t_next - T)
    return dict(init=init, Lx=s["Lx"], Ly=s["Ly"], N=s["N"], T=T, t_obs=t_obs, ncoll=ncoll,
                pairs=np.sort(np.stack([tr["i"][:ncoll], tr["j"][:ncoll]], 1), axis=1))


@pytest.fixture(scope="module")
def setup(edmd, oracle):
    return make_setup(edmd, oracle, NCOLL)


@pytest.fixture(scope="module")
def setup_short(edmd, oracle):
    """300 collisions: short enough that +-eps along a random 4N direction keeps
    the collision sequence of this chaotic system."""
    return make_setup(edmd, oracle, 300)


def engine(edmd, setup):
    desc = edmd.default_desc(setup["N"], setup["Lx"], setup["Ly"])
    sysd = dict(desc=desc, vr=None, **{k: setup["init"][k] for k in ("x", "y", "vx", "vy", "rad", "m")})
    return edmd.Engine([sysd])


def oracle_state_at(oracle, setup, arrays):
    """Run the oracle from `arrays` to t_obs; state flown to t_obs."""
    o = oracle.Oracle(arrays=arrays, Lx=setup["Lx"], Ly=setup["Ly"])
    tr, n = o.run(10 ** 9, t_stop=setup["t_obs"])
    pairs = np.sort(np.stack([tr["i"], tr["j"]], 1), axis=1)
    same = n == setup["ncoll"] and np.array_equal(pairs, setup["pairs"])
    st = o.state()
    t = setup["t_obs"]
    out = np.stack([st["x"] + st["vx"] * (t - st["tl"]), st["y"] + st["vy"] * (t - st["tl"]),
                    st["vx"], st["vy"]], 1)
    return out, same


def perturbed(setup, d, sign):
    a = {k: setup["init"][k].copy() for k in setup["init"]}
    for c, k in enumerate(("x", "y", "vx", "vy")):
        a[k] = a[k] + sign * EPS * d[:, c]
    return a


def min_image(setup, dpos):
    out = dpos.copy()
    out[:, 0] -= setup["Lx"] * np.round(out[:, 0] / setup["Lx"])
    out[:, 1] -= setup["Ly"] * np.round(out[:, 1] / setup["Ly"])
    return out


def msd_of(setup, pos, init=None):
    init = setup["init"] if init is None else init
    u = min_image(setup, pos - np.stack([init["x"], init["y"]], 1))
    u -= u.mean(0)
    return (u * u).sum() / setup["N"]


def test_tangent_matches_central_differences(edmd, oracle, setup_short):
    """A random direction in all four components of 64 disks."""
    setup = setup_short
    N = setup["N"]
    for seed in (3, 4, 5):
        rng = np.random.default_rng(seed)
        d = np.zeros((N, 4))
        d[rng.choice(N, 64, replace=False)] = rng.normal(size=(64, 4))
        sp, okp = oracle_state_at(oracle, setup, perturbed(setup, d, +1))
        sm, okm = oracle_state_at(oracle, setup, perturbed(setup, d, -1))
        if okp and okm:
            break
    assert okp and okm, "the perturbation changed the collision sequence"
    eng = engine(edmd, setup)
    vec, _ = eng.tangent(1, setup["ncoll"], vectors=d[None])
    T = eng.counters(0)["t"]
    assert T == setup["T"]                        # the GPU run is the oracle's run
    tan = vec[0].copy()
    tan[:, 0] += tan[:, 2] * (setup["t_obs"] - T)
    tan[:, 1] += tan[:, 3] * (setup["t_obs"] - T)
    diff = sp - sm
    diff[:, :2] = min_image(setup, diff[:, :2])
    fd = diff / (2 * EPS)
    rel = np.linalg.norm(tan - fd) / np.linalg.norm(fd)
    assert rel < 1e-5, rel


def test_adjoint_gradient_matches_central_differences(edmd, oracle, setup):
    N = setup["N"]
    eng = engine(edmd, setup)
    msd, g = eng.msd_gradient(NCOLL, ckpt_every=250, t_obs=setup["t_obs"])
    base, ok = oracle_state_at(oracle, setup, setup["init"])
    assert ok
    assert abs(msd - msd_of(setup, base[:, :2])) < 1e-12 * max(1.0, msd)
    rng = np.random.default_rng(7)
    checked = 0
    for k in rng.choice(N, 6, replace=False):
        for c, key in ((0, "x"), (1, "y"), (2, "vx"), (3, "vy")):
            d = np.zeros((N, 4))
            d[k, c] = 1.0
            ap, am = perturbed(setup, d, +1), perturbed(setup, d, -1)
            sp, okp = oracle_state_at(oracle, setup, ap)
            sm, okm = oracle_state_at(oracle, setup, am)
            if not (okp and okm):
                continue
            # the displacement is measured from the perturbed initial positions
            fd = (msd_of(setup, sp[:, :2], ap) - msd_of(setup, sm[:, :2], am)) / (2 * EPS)
            assert abs(g[key][k] - fd) <= 1e-6 * abs(fd) + 1e-9, (k, key, g[key][k], fd)
            checked += 1
    assert checked >= 12


def test_duality_with_oracle_displacement(edmd, oracle, setup):
    N = setup["N"]
    d = np.random.default_rng(9).normal(size=(N, 4))
    eng = engine(edmd, setup)
    vec, _ = eng.tangent(1, NCOLL, vectors=d[None])
    T = eng.counters(0)["t"]
    tan = vec[0].copy()
    tan[:, 0] += tan[:, 2] * (setup["t_obs"] - T)
    tan[:, 1] += tan[:, 3] * (setup["t_obs"] - T)
    base, _ = oracle_state_at(oracle, setup, setup["init"])
    u = min_image(setup, base[:, :2] - np.stack([setup["init"]["x"], setup["init"]["y"]], 1))
    u -= u.mean(0)
    # d u = d r(t_obs) - d r(0)
    dmsd_tangent = (2.0 / N) * (u * (tan[:, :2] - d[:, :2])).sum()
    eng2 = engine(edmd, setup)
    _, g = eng2.msd_gradient(NCOLL, ckpt_every=200, t_obs=setup["t_obs"])
    adj = np.stack([g["x"], g["y"], g["vx"], g["vy"]], 1)
    dmsd_adjoint = (adj * d).sum()
    assert abs(dmsd_adjoint - dmsd_tangent) <= 1e-9 * abs(dmsd_tangent)


def test_lyapunov_spectrum_32_vectors(edmd, setup):
    """Config 4: 32 tangent vectors, re-orthonormalised every 100 collisions."""
    eng = engine(edmd, setup)
    _, lam = eng.tangent(32, 10000, qr_every=100, seed=17)
    eng2 = engine(edmd, setup)
    _, lam2 = eng2.tangent(32, 10000, qr_every=100, seed=17)
    assert np.array_equal(lam, lam2)                  # deterministic
    assert np.isfinite(lam).all()
    assert lam[0] > 0.1                               # chaotic: positive leading exponent
    assert np.all(np.diff(lam) < 0.05 * abs(lam[0]))  # ordered (up to statistical noise)


def test_checkpoint_restore_replays_identically(edmd, setup):
    eng = engine(edmd, setup)
    eng.advance(max_coll=500)
    eng.checkpoint_save(0)
    L = edmd.load()
    L.edmd_set_log_capacity(eng.h, 4096)
    L.edmd_clear_log(eng.h)
    eng.advance(max_coll=2000, flags=edmd.F_LOG)
    a = eng.log(0)
    eng.checkpoint_restore(0)
    L.edmd_clear_log(eng.h)
    eng.advance(max_coll=2000, flags=edmd.F_LOG)
    b = eng.log(0)
    assert len(a) == 2000 and a.tobytes() == b.tobytes()


def test_torch_autograd_wrapper(edmd, oracle, setup):
    """torch.autograd.Function over the adjoint (check harness only)."""
    torch = pytest.importorskip("torch")
    from autograd_edmd import MeanSquareDisplacement
    N = setup["N"]
    vx = torch.tensor(setup["init"]["vx"], dtype=torch.float64, requires_grad=True)
    vy = torch.tensor(setup["init"]["vy"], dtype=torch.float64, requires_grad=True)
    f = MeanSquareDisplacement(edmd, setup["init"], setup["Lx"], setup["Ly"], NCOLL, setup["t_obs"])
    loss = f(vx, vy)
    loss.backward()
    k = 17
    d = np.zeros((N, 4))
    d[k, 2] = 1.0
    sp, okp = oracle_state_at(oracle, setup, perturbed(setup, d, +1))
    sm, okm = oracle_state_at(oracle, setup, perturbed(setup, d, -1))
    assert okp and okm
    fd = (msd_of(setup, sp[:, :2]) - msd_of(setup, sm[:, :2])) / (2 * EPS)
    assert abs(vx.grad[k].item() - fd) <= 1e-6 * abs(fd) + 1e-9


def cpu_tangent_spectrum(log, m, T, tl, qr_every):
    """CPU restatement of the tangent map of the collision log (the same
    Dellago-Posch-Hoover formulas as the engine: free flight to the contact,
    then the collision map) with CholQR2 re-orthonormalisation after every
    qr_every collisions at the time of the last one; T is [N][4][K] at the
    per-disk times tl.  Returns the accumulated log R_kk."""
    K = T.shape[2]
    logdiag = np.zeros(K)

    def qr(tq):
        nonlocal T
        Y = T.copy()
        Y[:, 0] += Y[:, 2] * (tq - tl)[:, None]
        Y[:, 1] += Y[:, 3] * (tq - tl)[:, None]
        tl[:] = tq
        Y = Y.reshape(-1, K)
        for _ in range(2):
            R = np.linalg.cholesky(Y.T @ Y).T
            logdiag[:] += np.log(np.diag(R))
            Y = Y @ np.linalg.inv(R)
        T = Y.reshape(-1, 4, K)

    for n, L in enumerate(log):
        i, j, t = int(L["i"]), int(L["j"]), float(L["t"])
        dx, dy, dvx, dvy, f = (float(L[k]) for k in ("dx", "dy", "dvx", "dvy", "f"))
        mi, mj = m[i], m[j]
        xi = T[i, 0] + T[i, 2] * (t - tl[i]); yi = T[i, 1] + T[i, 3] * (t - tl[i])
        xj = T[j, 0] + T[j, 2] * (t - tl[j]); yj = T[j, 1] + T[j, 3] * (t - tl[j])
        vxi, vyi, vxj, vyj = T[i, 2].copy(), T[i, 3].copy(), T[j, 2].copy(), T[j, 3].copy()
        rv = dx * dvx + dy * dvy
        drx, dry, ddvx, ddvy = xj - xi, yj - yi, vxj - vxi, vyj - vyi
        dtc = -(dx * drx + dy * dry) / rv
        rcx, rcy = drx + dvx * dtc, dry + dvy * dtc
        df = (f / rv) * (dvx * rcx + dvy * rcy + dx * ddvx + dy * ddvy)
        wx, wy = df * dx + f * rcx, df * dy + f * rcy
        T[i, 0] = xi - f * mj * dx * dtc; T[i, 1] = yi - f * mj * dy * dtc
        T[j, 0] = xj + f * mi * dx * dtc; T[j, 1] = yj + f * mi * dy * dtc
        T[i, 2] = vxi + mj * wx; T[i, 3] = vyi + mj * wy
        T[j, 2] = vxj - mi * wx; T[j, 3] = vyj - mi * wy
        tl[i] = tl[j] = t
        if (n + 1) % qr_every == 0:
            qr(t)
    return logdiag


def test_lyapunov_spectrum_pinned_to_cpu_restatement(edmd, oracle, setup):
    """Config 4's spectrum (32 vectors, CholQR2 every 100 collisions, 10^4
    collisions) against the CPU restatement of the tangent map applied to the
    collision log of the same run; the log's collisions are first checked
    against the oracle's (the reference's) sequence."""
    N, K, M, Q = setup["N"], 32, 10000, 100
    eng = engine(edmd, setup)
    L = edmd.load()
    L.edmd_set_log_capacity(eng.h, M + 16)
    L.edmd_clear_log(eng.h)
    eng.advance(max_coll=M, flags=edmd.F_LOG)
    log = eng.log(0, cap=M + 16)
    eng.close()
    assert len(log) == M
    o = oracle.Oracle(arrays=setup["init"], Lx=setup["Lx"], Ly=setup["Ly"])
    tr, n = o.run(M)
    assert n == M
    np.testing.assert_array_equal(log["t"], tr["t"])
    np.testing.assert_array_equal(log["i"], tr["i"])
    np.testing.assert_array_equal(log["j"], tr["j"])
    rng = np.random.default_rng(23)
    V = rng.normal(size=(K, N, 4))
    eng = engine(edmd, setup)
    _, lam = eng.tangent(K, M, qr_every=Q, vectors=V)
    T_end = eng.counters(0)["t"]
    eng.close()
    assert T_end == log["t"][-1]
    ld = cpu_tangent_spectrum(log, setup["init"]["m"], np.ascontiguousarray(V.transpose(1, 2, 0)),
                              np.zeros(N), Q)
    lam_cpu = ld / T_end
    assert np.all(np.abs(lam - lam_cpu) <= 1e-8 * np.abs(lam_cpu).max()), np.abs(lam - lam_cpu).max()


def test_duality_over_ten_thousand_collisions(edmd, setup):
    """Config 4's run length: the adjoint gradient (checkpoints every 500
    collisions, each segment recomputed) and the tangent map agree on
    d MSD along a random direction after 10^4 collisions."""
    N, M = setup["N"], 10000
    d = np.random.default_rng(29).normal(size=(N, 4))
    eng = engine(edmd, setup)
    vec, _ = eng.tangent(1, M, vectors=d[None])
    T = eng.counters(0)["t"]
    eng.sync()                                       # positions at T
    st = eng.state(0)
    eng.close()
    eng2 = engine(edmd, setup)
    msd, g = eng2.msd_gradient(M, ckpt_every=500)
    assert eng2.counters(0)["t"] == T
    eng2.close()
    u = min_image(setup, np.stack([st["x"], st["y"]], 1) -
                  np.stack([setup["init"]["x"], setup["init"]["y"]], 1))
    u -= u.mean(0)
    dmsd_tangent = (2.0 / N) * (u * (vec[0][:, :2] - d[:, :2])).sum()
    adj = np.stack([g["x"], g["y"], g["vx"], g["vy"]], 1)
    assert abs((adj * d).sum() - dmsd_tangent) <= 1e-8 * abs(dmsd_tangent)


def batch_setups(edmd, oracle, seeds=(11, 12, 13, 14)):
    """Replicas of config 4 with their own seeds, each 2000 collisions from the lattice."""
    out = []
    for sd in seeds:
        s = edmd.hex_start(1024, 0.60, sd)
        o = oracle.Oracle(arrays={k: s[k] for k in ("x", "y", "vx", "vy", "rad", "m", "type")},
                          Lx=s["Lx"], Ly=s["Ly"])
        o.run(2000, cap=1)
        o.sync()
        st = o.state()
        out.append(dict(desc=edmd.default_desc(s["N"], s["Lx"], s["Ly"]), vr=None,
                        **{k: st[k].copy() for k in ("x", "y", "vx", "vy", "rad", "m")}))
    return out


def test_batched_tangent_matches_single_systems(edmd, oracle):
    systems = batch_setups(edmd, oracle)
    eng = edmd.Engine(systems)
    lam = eng.tangent_batch(8, 1000, 100, seed=40)
    eng.close()
    for s, sysd in enumerate(systems):
        e1 = edmd.Engine([sysd])
        _, l1 = e1.tangent(8, 1000, qr_every=100, seed=40 + s)
        e1.close()
        np.testing.assert_allclose(lam[s], l1, rtol=1e-9, atol=1e-9 * np.abs(l1).max())


def test_batched_adjoint_matches_single_systems(edmd, oracle):
    systems = batch_setups(edmd, oracle)
    eng = edmd.Engine(systems)
    msd, g = eng.msd_gradient_batch(1000, ckpt_every=250)
    eng.close()
    off = np.cumsum([0] + [s["desc"].N for s in systems])
    for s, sysd in enumerate(systems):
        e1 = edmd.Engine([sysd])
        m1, g1 = e1.msd_gradient(1000, ckpt_every=250)
        e1.close()
        assert abs(msd[s] - m1) <= 1e-12 * m1
        for k in ("vx", "vy", "x", "y"):
            a, b = g[k][off[s]:off[s + 1]], g1[k]
            np.testing.assert_allclose(a, b, rtol=1e-9, atol=1e-9 * np.abs(b).max())
