"""Adjoint of a frozen-pair window (sqdem_adj_*) against central finite differences.

The reference for the finite differences is the oracle run as the same window (collider off,
no bound-separation erase, Ip2 coefficients refreshed from the perturbed materials with the
force history kept).  A finite difference is only a valid check when the +h and -h runs take
the same branches as the base run (Levenberg-Marquardt decisions, contact gates, Coulomb cap,
damping signs): both engines return a signature of their branches and the comparison uses the
directions whose three signatures agree.  Steps: h = 3e-5 (relative) for friction and
stiffness, whose losses are smooth but carry rounding noise of ~1e-11 relative, and h = 3e-8
for the exponents, where larger steps change the number of Levenberg-Marquardt iterations of
some pair.  Tolerance: 1e-5 relative on the directional derivative.
"""
import numpy as np
import pytest

from adjoint_scene import compressed_specimen, lid_weights, oracle_window, params_of

NSTEPS = 60
TOL = 1e-5
H_SMOOTH, H_EPS = 3e-5, 3e-8


@pytest.fixture(scope="module")
def scene():
    return compressed_specimen()


def _dirs(rng, spec, eps, mu, Kn, Ks):
    """One seeded direction per parameter kind with its finite-difference step."""
    part = (spec.kind == 0)[:, None]
    dE = rng.normal(size=eps.shape) * eps * part
    return [("eps", (dE, 0 * mu, 0 * Kn, 0 * Ks), H_EPS),
            ("mu", (0 * eps, rng.normal(size=mu.shape) * mu, 0 * Kn, 0 * Ks), H_SMOOTH),
            ("Kn", (0 * eps, 0 * mu, rng.normal(size=Kn.shape) * Kn, 0 * Ks), H_SMOOTH),
            ("Ks", (0 * eps, 0 * mu, 0 * Kn, rng.normal(size=Ks.shape) * Ks), H_SMOOTH)]


def _ad(gr, d):
    dE, dmu, dKn, dKs = d
    return float(np.sum(gr["eps"] * dE) + np.sum(gr["mu"] * dmu) + np.sum(gr["Kn"] * dKn) + np.sum(gr["Ks"] * dKs))


# ---------------------------------------------------------------------------- CPU (oracle)
def test_oracle_frozen_window_keeps_pair_set(scene):
    import oracle as O
    spec, bodies, recs = scene
    o = O.OracleScene.from_spec(spec)
    o.set_bodies(bodies)
    o.set_interactions(recs)
    runs0 = o.scalars()[7]
    o.set_frozen(True)
    o.step(150)
    after = o.interactions()
    assert o.scalars()[7] == runs0                      # no collider pass
    key = lambda r: (min(r[0], r[1]), max(r[0], r[1]))  # noqa: E731
    assert sorted(map(key, after[:, 0:2].tolist())) == sorted(map(key, recs[:, 0:2].tolist()))


def test_oracle_reset_phys_refreshes_coefficients_and_keeps_history(scene):
    import oracle as O
    spec, bodies, recs = scene
    o = O.OracleScene.from_spec(spec)
    o.set_bodies(bodies)
    o.set_interactions(recs)
    for m in range(spec.n_bodies):
        o.set_material(m, 2e5, 1e5, np.arctan(0.25))
    o.reset_phys()
    r = o.interactions()
    real = r[:, 2] != 0
    assert np.any(real)
    assert np.all(r[real, 23] == 2e5) and np.all(r[real, 24] == 1e5)
    assert np.allclose(r[real, 25], 0.25, rtol=1e-15)
    assert np.array_equal(r[:, 29:32], recs[:, 29:32])   # shear springs kept


def test_oracle_window_is_differentiable_along_friction(scene):
    """The oracle's window loss is smooth along friction: two step sizes with unchanged
    branches give the same central difference."""
    spec, bodies, recs = scene
    eps, mu, Kn, Ks = params_of(spec)
    wF, wX = lid_weights(spec.n_bodies), np.zeros((spec.n_bodies, 3))
    L0, s0, _ = oracle_window(spec, bodies, recs, eps, mu, Kn, Ks, NSTEPS, wF, wX)
    assert L0 != 0
    rng = np.random.default_rng(4)
    agreed = 0
    for trial in range(4):
        dmu = rng.normal(size=mu.shape) * mu
        fds = []
        for h in (H_SMOOTH, H_SMOOTH / 3):
            Lp, sp, _ = oracle_window(spec, bodies, recs, eps, mu + h * dmu, Kn, Ks, NSTEPS, wF, wX)
            Lm, sm, _ = oracle_window(spec, bodies, recs, eps, mu - h * dmu, Kn, Ks, NSTEPS, wF, wX)
            fds.append((Lp - Lm) / (2 * h) if sp == sm == s0 else None)
        if None in fds:
            continue
        assert abs(fds[0] - fds[1]) <= 1e-5 * abs(fds[0])
        agreed += 1
    assert agreed >= 2


def test_window_spec_checks_reject_unmodelled_scenes(scene):
    import copy
    from sudodem_gb300 import assemblies
    from sudodem_gb300.adjoint import check_window_spec
    spec = scene[0]
    check_window_spec(spec)
    bad = copy.deepcopy(spec)
    bad.info["periodic"] = True
    with pytest.raises(ValueError):
        check_window_spec(bad)
    bad = copy.deepcopy(spec)
    bad.materials["betan"] = np.full(len(bad.materials["betan"]), 0.1)
    with pytest.raises(ValueError):
        check_window_spec(bad)
    with pytest.raises(ValueError):
        check_window_spec(assemblies.hertz_mindlin(assemblies.walled_lattice(8, seed=1)))
    bad = copy.deepcopy(spec)
    bad.isSphere = bad.isSphere.copy()
    bad.isSphere[6] = 1
    with pytest.raises(ValueError):
        check_window_spec(bad)


# ---------------------------------------------------------------------------- GPU
@pytest.fixture(scope="module")
def window(scene):
    from sudodem_gb300.adjoint import AdjointWindow
    spec, bodies, recs = scene
    w = AdjointWindow(0)
    w.load(spec, bodies, recs)
    yield w
    w.close()


def _gpu_loss(w, spec, eps, mu, Kn, Ks, wF, wX, nsteps=NSTEPS, every=25):
    w.set_materials(Kn, Ks, mu)
    w.set_eps(eps)
    return w.forward(nsteps, every, wF, wX)


@pytest.mark.gpu
def test_adjoint_forward_matches_oracle(scene, window):
    spec, bodies, recs = scene
    eps, mu, Kn, Ks = params_of(spec)
    n = spec.n_bodies
    wF, wX = lid_weights(n), np.zeros((n, 3))
    for nsteps in (1, 20):
        L, _ = _gpu_loss(window, spec, eps, mu, Kn, Ks, wF, wX, nsteps, 10)
        Lo, _, ob = oracle_window(spec, bodies, recs, eps, mu, Kn, Ks, nsteps, wF, wX)
        st = window.state()
        assert abs(L - Lo) <= 1e-9 * abs(Lo)
        assert np.max(np.abs(st[:, 0:3] - ob[:, 0:3])) <= 1e-12
        assert np.max(np.abs(st[:, 3:7] - ob[:, 3:7])) <= 1e-10
        assert np.max(np.abs(st[:, 7:10] - ob[:, 7:10])) <= 1e-9 * max(1.0, np.max(np.abs(ob[:, 7:10])))


@pytest.mark.gpu
@pytest.mark.parametrize("reference", ["gpu", "oracle"])
def test_adjoint_gradient_matches_central_differences(scene, window, reference):
    spec, bodies, recs = scene
    eps, mu, Kn, Ks = params_of(spec)
    n = spec.n_bodies
    wF, wX = lid_weights(n), np.zeros((n, 3))
    L0, sg0 = _gpu_loss(window, spec, eps, mu, Kn, Ks, wF, wX)
    gr = window.backward()
    assert window.report()["replay_mismatches"] == 0
    assert L0 != 0
    if reference == "oracle":
        L0o, sg0, _ = oracle_window(spec, bodies, recs, eps, mu, Kn, Ks, NSTEPS, wF, wX)
        assert abs(L0o - L0) <= 1e-8 * abs(L0)
    rng = np.random.default_rng(11)
    checked = {}
    for trial in range(4):
        for name, d, h in _dirs(rng, spec, eps, mu, Kn, Ks):
            dE, dmu, dKn, dKs = d
            vals, sigs = [], []
            for s in (1, -1):
                args = (eps + s * h * dE, mu + s * h * dmu, Kn + s * h * dKn, Ks + s * h * dKs)
                if reference == "gpu":
                    l, sg = _gpu_loss(window, spec, *args, wF, wX)
                else:
                    l, sg, _ = oracle_window(spec, bodies, recs, *args, NSTEPS, wF, wX)
                vals.append(l)
                sigs.append(sg)
            if not (sigs[0] == sigs[1] == sg0):
                continue
            fd = (vals[0] - vals[1]) / (2 * h)
            ad = _ad(gr, d)
            assert abs(fd - ad) <= TOL * abs(ad), (name, trial, fd, ad)
            checked[name] = checked.get(name, 0) + 1
    assert all(checked.get(k, 0) >= 2 for k in ("eps", "mu", "Kn", "Ks")), checked


@pytest.mark.gpu
def test_forced_branches_central_differences_at_the_relative_step_1e_6(scene, window):
    """The branch tape (sqdem_adj_set_branches) on the GPU: a forced run with the recorded
    parameters is bitwise the recorded one, and central differences at the relative step 1e-6
    of runs forced onto the recorded branches match the reverse pass along 20 seeded directions
    within 1e-5 relative, or within the loss's measured rounding noise divided by h where the
    directional derivative is too small for the difference to resolve it (at least 15 of 20
    within 1e-5), while naturally evaluated runs leave the recorded branches in some of them."""
    from sudodem_gb300.adjoint import AdjointWindow
    spec, bodies, recs = scene
    eps, mu, Kn, Ks = params_of(spec)
    n = spec.n_bodies
    wF, wX = lid_weights(n), np.zeros((n, 3))
    w = window
    h = 1e-6
    try:
        w.set_branches(AdjointWindow.BRANCH_RECORD)
        L0, s0 = _gpu_loss(w, spec, eps, mu, Kn, Ks, wF, wX)
        gr = w.backward()
        rec = w.branch_report()
        assert rec["decisions"] > 0 and rec["disagreements"] == 0 and rec["steps_recorded"] == NSTEPS
        w.set_branches(AdjointWindow.BRANCH_FORCE)
        L1, s1 = _gpu_loss(w, spec, eps, mu, Kn, Ks, wF, wX)
        rep = w.branch_report()
        assert L1 == L0 and s1 == s0 and rep["disagreements"] == 0 and rep["decisions"] == rec["decisions"]
        rng = np.random.default_rng(7)
        noise = 0.0
        for k in range(4):
            d = rng.normal(size=mu.shape) * mu
            Ls, _ = _gpu_loss(w, spec, eps, mu + 1e-13 * d, Kn, Ks, wF, wX)
            noise = max(noise, abs(Ls - L0 - 1e-13 * float(np.sum(gr["mu"] * d))))
        part = (spec.kind == 0)[:, None]
        within, left = 0, 0
        for trial in range(5):
            dirs = [("eps", (rng.normal(size=eps.shape) * eps * part, 0 * mu, 0 * Kn, 0 * Ks)),
                    ("mu", (0 * eps, rng.normal(size=mu.shape) * mu, 0 * Kn, 0 * Ks)),
                    ("Kn", (0 * eps, 0 * mu, rng.normal(size=Kn.shape) * Kn, 0 * Ks)),
                    ("Ks", (0 * eps, 0 * mu, 0 * Kn, rng.normal(size=Ks.shape) * Ks))]
            for name, d in dirs:
                dE, dmu, dKn, dKs = d
                vals, dis = [], 0
                for sg in (1, -1):
                    l, _ = _gpu_loss(w, spec, eps + sg * h * dE, mu + sg * h * dmu, Kn + sg * h * dKn,
                                     Ks + sg * h * dKs, wF, wX)
                    vals.append(l)
                    dis += w.branch_report()["disagreements"]
                left += dis > 0
                fd = (vals[0] - vals[1]) / (2 * h)
                ad = _ad(gr, d)
                within += abs(fd - ad) <= TOL * abs(ad)
                assert abs(fd - ad) <= TOL * abs(ad) + 2 * noise / h, (name, trial, fd, ad, dis, noise)
        assert within >= 15 and left > 0, (within, left)
    finally:
        w.set_branches(AdjointWindow.BRANCH_NATURAL)
        w.set_materials(Kn, Ks, mu)
        w.set_eps(eps)


@pytest.mark.gpu
def test_adjoint_checkpoint_interval_changes_nothing(scene, window):
    spec, bodies, recs = scene
    eps, mu, Kn, Ks = params_of(spec)
    n = spec.n_bodies
    wF = lid_weights(n)
    wX = np.random.default_rng(2).normal(size=(n, 3)) * (spec.kind == 0)[:, None]
    res = []
    for every in (1, 7, 60, NSTEPS):
        L, sg = _gpu_loss(window, spec, eps, mu, Kn, Ks, wF, wX, NSTEPS, every)
        st = window.state()
        g = window.backward()
        assert np.array_equal(window.state(), st)   # the reverse pass leaves the window's result readable
        res.append((L, sg, g))
    for L, sg, g in res[1:]:
        assert L == res[0][0] and sg == res[0][1]
        for k in g:
            assert np.array_equal(g[k], res[0][2][k]), k


@pytest.mark.gpu
def test_replay_shapes_agree_bitwise(scene, window):
    spec, bodies, recs = scene
    eps, mu, Kn, Ks = params_of(spec)
    n = spec.n_bodies
    wF = lid_weights(n)
    wX = np.random.default_rng(3).normal(size=(n, 3)) * (spec.kind == 0)[:, None]
    res = []
    for shape, blocks in ((0, 1), (1, 1), (2, 1), (3, 1), (3, 0), (3, 2), (1, 0)):
        window.set_replay(shape)
        window.set_replay_blocks(blocks)   # resident blocks per SM of the grouped kernels
        _gpu_loss(window, spec, eps, mu, Kn, Ks, wF, wX)
        res.append(window.backward())
        assert window.report()["replay_mismatches"] == 0
    window.set_replay(3)
    window.set_replay_blocks(1)
    for r in res[1:]:
        for k in r:
            assert np.array_equal(res[0][k], r[k]), k


@pytest.mark.gpu
def test_cooperative_forward_is_bitwise_the_single_thread_one(scene, window):
    spec, bodies, recs = scene
    eps, mu, Kn, Ks = params_of(spec)
    n = spec.n_bodies
    wF = lid_weights(n)
    wX = np.random.default_rng(5).normal(size=(n, 3)) * (spec.kind == 0)[:, None]
    res = []
    for coop in (True, False):
        window.set_forward(coop)
        L, sg = _gpu_loss(window, spec, eps, mu, Kn, Ks, wF, wX)
        st = window.state()
        g = window.backward()
        assert window.report()["replay_mismatches"] == 0
        res.append((L, sg, st, g))
    window.set_forward(True)
    (L0, s0, st0, g0), (L1, s1, st1, g1) = res
    assert L0 == L1 and s0 == s1 and np.array_equal(st0, st1)
    for k in g0:
        assert np.array_equal(g0[k], g1[k]), k


@pytest.mark.gpu
def test_window_loss_torch_autograd(scene, window):
    torch = pytest.importorskip("torch")
    from sudodem_gb300.adjoint import window_loss
    spec, bodies, recs = scene
    eps, mu, Kn, Ks = params_of(spec)
    n = spec.n_bodies
    wF, wX = lid_weights(n), np.zeros((n, 3))
    te = torch.tensor(eps, dtype=torch.float64, requires_grad=True)
    tm = torch.tensor(mu, dtype=torch.float64, requires_grad=True)
    tkn = torch.tensor(Kn, dtype=torch.float64, requires_grad=True)
    tks = torch.tensor(Ks, dtype=torch.float64, requires_grad=True)
    loss = window_loss(window, te, tm, tkn, tks, NSTEPS, 25, wF, wX)
    (2.0 * loss).backward()
    L, _ = _gpu_loss(window, spec, eps, mu, Kn, Ks, wF, wX)
    g = window.backward()
    assert float(loss.detach()) == L
    assert np.array_equal(te.grad.numpy(), 2.0 * g["eps"])
    assert np.array_equal(tm.grad.numpy(), 2.0 * g["mu"])
    assert np.array_equal(tkn.grad.numpy(), 2.0 * g["Kn"])
    assert np.array_equal(tks.grad.numpy(), 2.0 * g["Ks"])


@pytest.mark.gpu
def test_adjoint_window_from_engine_records(scene):
    """A window started from the GPU engine's own records (after ten ordinary engine steps)
    follows the oracle's window from the same records."""
    from sudodem_gb300 import Engine
    from sudodem_gb300.adjoint import AdjointWindow
    spec, bodies, recs = scene
    import oracle as O
    orc = O.OracleScene.from_spec(spec)
    orc.set_bodies(bodies)
    orc.set_interactions(recs)
    eng = Engine(device=0)
    eng.load(spec)
    eng.put_body_state(orc.bodies())
    eng.put_interactions(orc.interactions())
    eng.put_scalars(orc.scalars())
    eng.step(10)
    eng.sync()
    st, er = eng.body_state(), eng.interactions(include_potential=True)
    eng.close()
    w = AdjointWindow(0)
    w.load(spec, st, er)
    eps, mu, Kn, Ks = params_of(spec)
    n = spec.n_bodies
    wF, wX = lid_weights(n), np.zeros((n, 3))
    L, _ = w.forward(20, 5, wF, wX)
    Lo, _, ob = oracle_window(spec, st, er, eps, mu, Kn, Ks, 20, wF, wX)
    assert np.max(np.abs(w.state()[:, 0:3] - ob[:, 0:3])) <= 1e-12
    assert abs(L - Lo) <= 1e-9 * abs(Lo)
    w.close()
