"""Edge cases of the superellipsoid timestep on the GPU, through the C ABI, against the oracle:
a scene without particles, one particle on the floor (wall contact only), two particles with
coincident centres (the narrowphase meets NaN angles), and the host-side limits."""
import numpy as np
import pytest

from oracle import OracleScene
from sudodem_gb300 import Engine, SqdemError, assemblies

pytestmark = pytest.mark.gpu


def _params(dt=2e-6):
    return {"dt": dt, "gravity": (0.0, 0.0, -9.81), "damping": 0.3, "verletDist": 2e-4, "targetInterv": 50,
            "minSweepDistFactor": 0.1, "sortAxis": 0, "isSuperquadrics": 1, "exactAsphericalRot": 1}


def _box(b, side=10e-3, lid=0.2):
    assemblies._add_wall(b, [0, 0, 0], 0, +1)
    assemblies._add_wall(b, [side, 0, 0], 0, -1)
    assemblies._add_wall(b, [0, 0, 0], 1, +1)
    assemblies._add_wall(b, [0, side, 0], 1, -1)
    assemblies._add_wall(b, [0, 0, 0], 2, +1)
    assemblies._add_wall(b, [0, 0, lid], 2, -1)


def _engine(spec):
    e = Engine(device=0)
    e.load(spec)
    return e


def test_scene_without_particles_steps(gpu):
    b = assemblies._builder()
    _box(b)
    spec = assemblies._finish(b, assemblies.default_material(), _params(), {"box": 10e-3})
    spec.state[5, 7:10] = (0.0, 0.0, -0.5)   # the lid moves down at its prescribed velocity
    eng, orc = _engine(spec), OracleScene.from_spec(spec)
    eng.step(10); rep = eng.sync(); orc.step(10)
    assert int(eng.scalars()[0]) == 10
    assert rep["lm_calls"] == 0 and rep["nan_forces"] == 0
    assert len(eng.interactions(False)) == 0
    g, r = eng.body_state(), orc.bodies()
    assert np.array_equal(g[:, 0:3], r[:, 0:3])
    assert g[5, 2] < 0.2


def test_one_particle_resting_on_the_floor(gpu):
    b = assemblies._builder()
    _box(b)
    assemblies._add_sq(b, [1e-3, 0.8e-3, 0.7e-3], [0.8, 1.2], assemblies._quat_normalize([1, 0.2, 0.1, 0]),
                       [5e-3, 5e-3, 0.9e-3], 2650.0)
    spec = assemblies._finish(b, assemblies.default_material(), _params(), {"box": 10e-3})
    eng, orc = _engine(spec), OracleScene.from_spec(spec)
    for _ in range(4):
        eng.step(500); eng.sync(); orc.step(500)
        g, r = eng.body_state(), orc.bodies()
        assert np.allclose(g[6, 0:16], r[6, 0:16], rtol=1e-9, atol=1e-15)
    assert 0 < g[6, 2] < 1e-3
    recs = eng.interactions(False)
    assert len(recs) >= 1 and np.all(recs[:, 0] == 4)   # the floor, as id1 (wall first)


def test_coincident_centres_do_not_break_the_step(gpu):
    spec = assemblies.pair_scene([1e-3, 0.9e-3, 0.8e-3, 0.7, 1.3], [0.9e-3, 0.9e-3, 0.9e-3, 1.1, 0.9],
                                 [0, 0, 0], [0, 0, 0], [1, 0, 0, 0], [0.9, 0.1, 0.3, 0.2])
    eng, orc = _engine(spec), OracleScene.from_spec(spec)
    eng.step(3); rep = eng.sync(); orc.step(3)
    g, r = eng.body_state(), orc.bodies()
    assert np.array_equal(np.isfinite(g[:, 0:16]), np.isfinite(r[:, 0:16]))
    assert np.all(np.isfinite(g[:, 0:3]))
    st = orc.stats()
    assert rep["nan_normals"] == st["nan_normals"]


def test_host_limits(gpu):
    b = assemblies._builder()
    for k in range(65):
        assemblies._add_wall(b, [0, 0, -1.0 - k], 2, +1)
    assemblies._add_sq(b, [1e-3, 1e-3, 1e-3], [1.0, 1.0], [1, 0, 0, 0], [0, 0, 0], 2650.0)
    spec = assemblies._finish(b, assemblies.default_material(), _params(), {})
    e = Engine(device=0)
    with pytest.raises(SqdemError) as ei:
        e.load(spec)
    assert ei.value.status == 3   # SQDEM_ERR_CAPACITY: at most 64 walls
    e2 = Engine(device=0)
    with pytest.raises(SqdemError):
        e2.step(1)                # bodies and materials first
