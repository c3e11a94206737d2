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
