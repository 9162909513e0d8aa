"""Start states of adjoint windows for the tests: a small walled specimen deposited by the oracle
with a lid driven down onto it (so that every kind of pair is present: particle-particle,
particle-wall, particle-lid, with shear-spring history), one material per body (per-particle
friction), and the oracle's frozen-pair window as the finite-difference reference."""
import math

import numpy as np

import oracle as O
from sudodem_gb300 import assemblies


def compressed_specimen(n=27, seed=2, relax_time=0.067, v_lid=0.1, mu_range=(0.3, 0.7)):
    """(spec, bodies, interactions): n superellipsoids deposited for `relax_time` seconds in an 8.2 mm
    box, then a lid moving down at v_lid (m/s) until it has carried a force for 200 steps in a
    row; per-body materials with friction coefficients uniform in mu_range."""
    spec = assemblies.walled_lattice(n, seed=seed, spacing=2.6e-3, per_side=3, box=8.2e-3, lid_height=0.2)
    nb = spec.n_bodies
    rng = np.random.default_rng(seed + 100)
    mu = rng.uniform(*mu_range, nb)
    m0 = spec.materials
    spec.materials = {k: np.full(nb, float(v[0])) for k, v in m0.items()}
    spec.materials["frictionAngle"] = np.arctan(mu)
    spec.mat = np.arange(nb, dtype=np.int32)
    o = O.OracleScene.from_spec(spec)
    b = o.bodies()
    b[6:, 2] -= 0.7e-3
    o.set_bodies(b)
    o.step(int(round(relax_time / spec.params["dt"])))
    b = o.bodies()
    part = spec.kind == 0
    b[5, 2] = np.max(b[part, 2] + np.max(spec.shape5[part, 0:3], axis=1)) + 0.05e-3
    b[5, 7:10] = [0.0, 0.0, -v_lid]
    o.set_bodies(b)
    held = 0
    for _ in range(int(round(0.1 / (10 * spec.params["dt"])))):   # at most 0.1 s of lid travel
        o.step(10)
        held = held + 1 if abs(o.bodies()[5, 18]) > 1e-3 else 0
        if held == 20:
            break
    return spec, o.bodies(), o.interactions()


def params_of(spec):
    m = spec.materials
    return (spec.shape5[:, 3:5].copy(), np.tan(np.asarray(m["frictionAngle"])), np.array(m["Kn"], dtype=float),
            np.array(m["Ks"], dtype=float))


def oracle_window(spec, bodies, recs, eps, mu, Kn, Ks, nsteps, wF, wX):
    """The oracle's frozen-pair window from the same start: (loss, branch signature, bodies)."""
    o = O.OracleScene.from_spec(spec)
    o.set_bodies(bodies)
    o.set_interactions(recs)
    for m in range(len(Kn)):
        o.set_material(m, Kn[m], Ks[m], math.atan(mu[m]))
    for i in range(spec.n_bodies):
        if spec.kind[i] == 0:
            o.set_eps(i, eps[i, 0], eps[i, 1])
    o.reset_phys()
    o.set_frozen(True)
    o.step(nsteps)
    b = o.bodies()
    loss = float(np.sum(wF * b[:, 16:19]) + np.sum(wX * b[:, 0:3]))
    sig = o.signature()
    o.close()
    return loss, sig, b


def lid_weights(n, lid=5):
    """Loss = normal force on the lid (its z force) of the window's last step."""
    w = np.zeros((n, 3))
    w[lid, 2] = 1.0
    return w
