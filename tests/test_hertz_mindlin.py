"""Hertz-Mindlin contact model: SuperquadricsGeom2 (Nelder-Mead closest points, principal
curvatures, contact ellipse), Ip2_SuperquadricsMat2_SuperquadricsMat2_HertzMindlinPhys and
SuperquadricsLaw2.

CPU: the oracle against closed forms (Hertz sphere law, Gaussian curvature of an ellipsoid,
the circular-contact limit of the ellipse fits) and against the Levenberg-Marquardt depth.
GPU: libsqdem_gpu.so through the C ABI against the oracle, with the tolerance stated against
the oracle's own one-ulp sensitivity (the Nelder-Mead search stops at a relative tolerance of
1e-3, so a last-ulp difference of CUDA's pow/atan2/sin/cos can change which simplex vertex a
search returns).
"""
import math

import numpy as np
import pytest

import oracle as O
from oracle import OracleScene
from sudodem_gb300 import Engine, assemblies

CURV = slice(47, 51)
ELL = slice(51, 55)


def sphere_pair(r1, r2, overlap, G=2e8, nu=0.3):
    spec = assemblies.pair_scene([r1, r1, r1, 1.0, 1.0], [r2, r2, r2, 1.0, 1.0], [0, 0, 0],
                                 [r1 + r2 - overlap, 0, 0], [1, 0, 0, 0], [1, 0, 0, 0])
    spec.isSphere[6:] = 1
    return assemblies.hertz_mindlin(spec, G=G, nu=nu)


def test_sphere_pair_is_hertz():
    r1, r2, d, G, nu = 1e-3, 0.7e-3, 2e-6, 2e8, 0.3
    orc = OracleScene.from_spec(sphere_pair(r1, r2, d, G, nu))
    orc.step(1)
    rec = [r for r in orc.interactions() if r[0] > 5][0]
    R = r1 * r2 / (r1 + r2)
    estar = G / (1 - nu)                          # E/(2(1-nu^2)) of two equal materials
    f_hertz = 4.0 / 3.0 * estar * math.sqrt(R) * d ** 1.5
    assert abs(rec[4] - d) < 1e-15
    assert rec[56] == 1 and abs(rec[55] - (r1 + r2) / (r1 * r2)) < 1e-9 * rec[55]
    assert abs(np.linalg.norm(rec[26:29]) - f_hertz) < 1e-12 * f_hertz


def test_curvatures_of_ellipsoid_match_gaussian_curvature():
    a, b, c = 1.5e-3, 1.0e-3, 0.7e-3
    for ph1 in (0.3, 1.0, -0.5):
        k, _, _, _ = O.curvatures([a, b, c, 1.0, 1.0], 1e-20, ph1)
        x, z = a * math.cos(ph1), c * math.sin(ph1)
        K = 1 / (a * a * b * b * c * c * (x * x / a ** 4 + z * z / c ** 4) ** 2)
        assert abs(k[0] * k[1] - K) < 1e-12 * K
    k, _, _, _ = O.curvatures([1e-3, 1e-3, 1e-3, 1.0, 1.0], 0.4, -0.2)
    assert np.allclose(k, [-1e3, -1e3], rtol=1e-7)   # sqrt(|H^2 - K|) of a rounding-level difference


def test_ellipse_fits_circular_limit():
    s, alpha, K, E = O.hertz_mindlin([-1e3, -1e3], [-2e3, -2e3], 0.0)
    assert s == 3e3 and alpha == 1.0
    assert abs(K - math.pi / 2) < 1e-7 and abs(E - math.pi / 2) < 1e-7
    s, alpha, K, E = O.hertz_mindlin([-1e3, -500], [-800, -300], 0.4)
    assert alpha > 1 and K > E > 1


def test_nelder_mead_depth_close_to_lm_depth():
    rng = np.random.default_rng(1)
    o = OracleScene()
    o.L.sqo_add_material(o.h, 1e5, 5e4, 0.5, 0, 0, 2650)
    rel = []
    for _ in range(30):
        r1, r2 = rng.uniform(0.8e-3, 1.2e-3, 3), rng.uniform(0.8e-3, 1.2e-3, 3)
        e1, e2 = rng.uniform(0.6, 1.4, 2), rng.uniform(0.6, 1.4, 2)
        q1, q2 = assemblies.random_quaternions(rng, 2)
        d = rng.standard_normal(3)
        d /= np.linalg.norm(d)
        ia = o.L.sqo_add_sq(o.h, *r1, *e1, 0, O._dp(np.ascontiguousarray(q1)), 0, O._dp(np.zeros(3)))
        ib = o.L.sqo_add_sq(o.h, *r2, *e2, 0, O._dp(np.ascontiguousarray(q2)), 0,
                            O._dp(np.ascontiguousarray(d * 1.6e-3)))
        lm, nm = o.pair_geom(ia, ib), o.pair_geom2(ia, ib)
        assert nm["depth"] > 0 and nm["nm_evaluations"] < 100
        warm = o.pair_geom2(ia, ib, prior=[*nm["contactAngle"], nm["depth"], 0])
        assert warm["nm_evaluations"] <= 30
        rel.append(abs(nm["depth"] - lm["depth"]) / lm["depth"])
    assert np.median(rel) < 0.01 and max(rel) < 0.05


def test_hm_oracle_runs_without_nan():
    spec = assemblies.hertz_mindlin(assemblies.walled_lattice(120, seed=2, box=14e-3, per_side=5))
    orc = OracleScene.from_spec(spec, threads=2)
    orc.step(1500)
    b = orc.bodies()
    assert np.all(np.isfinite(b[:, 0:16]))
    assert orc.nan_forces() == 0


# ---------------------------------------------------------------------------
# GPU against the oracle

def engine_for(spec, **kw):
    e = Engine(device=0, **kw)
    e.load(spec)
    return e


def by_pair(recs):
    return {(int(r[0]), int(r[1])): r for r in recs}


def touching_common(gi, ri):
    G, R = by_pair(gi), by_pair(ri)
    keys = [k for k, r in R.items() if k in G and r[4] > 0 and r[2] == 1]
    return np.array([G[k] for k in keys]), np.array([R[k] for k in keys])


def rel_force_errors(G, R):
    fg = G[:, 26:29] + G[:, 29:32]
    fr = R[:, 26:29] + R[:, 29:32]
    den = np.linalg.norm(fr, axis=1)
    return np.linalg.norm(fg - fr, axis=1) / np.where(den > 0, den, 1)


def snapshot_into(eng, orc):
    eng.put_body_state(orc.bodies())
    eng.put_interactions(orc.interactions())
    eng.put_scalars(orc.scalars())


def dense_hm(seed=5, n=400):
    return assemblies.hertz_mindlin(assemblies.walled_lattice(n, seed=seed, box=14e-3, per_side=5, spacing=2.1e-3))


def oracle_self_sensitivity(spec, state):
    a, b = OracleScene.from_spec(spec), OracleScene.from_spec(spec)
    bodies, intr, sc = state
    rng = np.random.default_rng(0)
    pert = bodies.copy()
    sgn = rng.choice([-1.0, 1.0], size=pert[:, 0:3].shape)
    pert[:, 0:3] = np.nextafter(pert[:, 0:3], pert[:, 0:3] + sgn * np.inf)
    for o, bb in ((a, bodies), (b, pert)):
        o.set_bodies(bb); o.set_interactions(intr); o.set_scalars(sc); o.rebuild_sorted_bounds()
        o.step(1)
    G, R = touching_common(b.interactions(), a.interactions())
    return rel_force_errors(G, R)


@pytest.mark.gpu
def test_gpu_sphere_pair_is_exact(gpu):
    spec = sphere_pair(1e-3, 0.7e-3, 2e-6)
    eng, orc = engine_for(spec), OracleScene.from_spec(spec)
    eng.set_record_full(True)
    eng.step(1); eng.sync(); orc.step(1)
    G, R = touching_common(eng.interactions(True), orc.interactions())
    assert len(G) == 1
    assert np.allclose(G[0], R[0], rtol=1e-14, atol=0)


@pytest.mark.gpu
def test_gpu_single_step_within_oracle_conditioning(gpu):
    spec = dense_hm(seed=5)
    orc = OracleScene.from_spec(spec, threads=4)
    orc.step(3)
    state = (orc.bodies(), orc.interactions(), orc.scalars())
    eng = engine_for(spec)
    eng.set_record_full(True)
    snapshot_into(eng, orc)
    eng.step(1); eng.sync(); orc.step(1)
    G, R = touching_common(eng.interactions(True), orc.interactions())
    assert len(G) > 50
    e = rel_force_errors(G, R)
    selfe = oracle_self_sensitivity(spec, state)
    q = lambda x, p: float(np.quantile(x, p))
    print(f"touching={len(e)} gpu-vs-oracle force err: median {q(e, .5):.2e} p90 {q(e, .9):.2e} max {e.max():.2e}; "
          f"oracle 1-ulp self: median {q(selfe, .5):.2e} p90 {q(selfe, .9):.2e} max {selfe.max():.2e}")
    assert q(e, 0.5) < 1e-9
    assert q(e, 0.9) < max(100 * q(selfe, 0.9), 1e-8)
    assert np.mean(e < 1e-6) > 0.95
    # the ellipse and stiffness of the contacts whose search ended at the same vertex
    same = np.all(G[:, 5:7] == R[:, 5:7], axis=1) & (G[:, 0] > 5)
    assert same.sum() > 0.9 * np.sum(G[:, 0] > 5)
    for sl in (CURV, ELL, slice(23, 25)):
        d = np.abs(G[same][:, sl] - R[same][:, sl]) / np.maximum(np.abs(R[same][:, sl]), 1e-300)
        assert np.median(d) < 1e-10


@pytest.mark.gpu
def test_gpu_wall_contacts_tight(gpu):
    spec = dense_hm(seed=8)
    orc = OracleScene.from_spec(spec, threads=4)
    orc.step(60)   # the lattice's initial overlaps throw particles against the walls
    eng = engine_for(spec)
    snapshot_into(eng, orc)
    eng.step(1); eng.sync(); orc.step(1)
    G, R = touching_common(eng.interactions(True), orc.interactions())
    wall = G[:, 0] < 6
    assert wall.sum() > 5
    assert rel_force_errors(G[wall], R[wall]).max() < 1e-11


@pytest.mark.gpu
def test_gpu_short_run_statistics_match_oracle(gpu):
    spec = assemblies.hertz_mindlin(assemblies.walled_lattice(300, seed=3))
    eng, orc = engine_for(spec), OracleScene.from_spec(spec, threads=8)
    eng.step(5000); eng.sync(); orc.step(5000)
    g, r = eng.body_state(), orc.bodies()
    p = 6
    assert abs(g[p:, 2].mean() - r[p:, 2].mean()) < 1e-6 * abs(r[p:, 2].mean())
    rep = eng.sync()
    assert rep["nan_forces"] == 0


@pytest.mark.gpu
def test_gpu_model_switch_and_moduli_roundtrip(gpu):
    spec = dense_hm(seed=4, n=200)
    eng = engine_for(spec)
    assert eng.contact_model() == "hertz_mindlin"
    G, nu = eng.material_moduli()
    assert G[0] == 2e8 and nu[0] == 0.3
    eng.step(30); eng.sync()
    blob = eng.snapshot()
    a = Engine(device=0)
    a.restore(blob)
    assert a.contact_model() == "hertz_mindlin"
    assert np.array_equal(a.material_moduli()[0], G)
    eng.step(30); a.step(30)
    eng.sync(); a.sync()
    assert np.array_equal(eng.body_state(), a.body_state())
    assert np.array_equal(eng.interactions(True), a.interactions(True))


@pytest.mark.gpu
def test_gpu_deterministic_and_graph_equals_eager(gpu):
    spec = dense_hm(seed=6, n=200)
    a, b, c = engine_for(spec), engine_for(spec), engine_for(spec, use_graph=False)
    for e in (a, b, c):
        e.step(50)
        e.sync()
    assert np.array_equal(a.body_state(), b.body_state())
    assert np.array_equal(a.interactions(True), b.interactions(True))
    assert np.array_equal(a.body_state(), c.body_state())


@pytest.mark.gpu
def test_gpu_cooperative_evaluations_change_nothing(gpu):
    """Drained warps evaluate the points the remaining searches may ask for next, with six
    lanes per point when few remain (set_lm_spread switches that off): bitwise the same
    results."""
    spec = dense_hm(seed=7, n=400)
    a, b = engine_for(spec), engine_for(spec)
    b.set_lm_spread(False)
    a.step(40); b.step(40)
    ra, rb = a.sync(), b.sync()
    assert np.array_equal(a.body_state(), b.body_state())
    assert np.array_equal(a.interactions(True), b.interactions(True))
    for k in ("lm_calls", "lm_iterations", "nan_forces"):
        assert ra[k] == rb[k], k
    assert ra["evals_fp64"] >= rb["evals_fp64"] > 0   # speculative points evaluated in spare slots


@pytest.mark.gpu
def test_gpu_periodic_cell_single_step(gpu):
    """Periodic cell: the Hertz-Mindlin geometry uses unshifted positions (only precompute sees
    shift2), as the reference; the GPU follows the oracle there too."""
    spec = assemblies.hertz_mindlin(assemblies.periodic_cell(400, seed=4, solid_fraction=0.42, strain_rate=3.0))
    orc = OracleScene.from_spec(spec, threads=1)
    orc.step(10)
    eng = engine_for(spec)
    snapshot_into(eng, orc)
    eng.put_cell(orc.cell())
    eng.step(1); eng.sync(); orc.step(1)
    assert np.array_equal(eng.cell(), orc.cell())
    G, R = touching_common(eng.interactions(True), orc.interactions())
    assert len(G) > 30
    e = rel_force_errors(G, R)
    assert np.median(e) < 1e-9 and np.mean(e < 1e-6) > 0.95


@pytest.mark.gpu
def test_gpu_precision_flag_does_not_change_the_hm_search(gpu):
    """The Hertz-Mindlin search always runs in FP64: a context created with the mixed form
    gives the same results bit for bit."""
    spec = dense_hm(seed=9, n=300)
    a, b = engine_for(spec), engine_for(spec, precision="mixed")
    a.step(25); b.step(25)
    a.sync(); b.sync()
    assert np.array_equal(a.body_state(), b.body_state())
    assert np.array_equal(a.interactions(True), b.interactions(True))
