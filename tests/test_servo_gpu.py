"""CompressionEngine, quiet flag and Shop reductions on the GPU against the CPU oracle.

The controller (pkg/dem/Compression.cpp:395-604) is checked one step at a time from a shared
state: the oracle runs the specimen, its bodies, interactions, collider scalars and engine
state are loaded into the GPU context, both take one step, and the wall positions and the
engine's state must agree to the precision of the force sums (their order differs: the
reference's and the oracle's container order against the GPU's table order).
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
from oracle import OracleScene  # noqa: E402
from sudodem_gb300 import Engine, assemblies  # noqa: E402
from sudodem_gb300.servo import STATE_NAMES, servo_config, state_dict  # noqa: E402

pytestmark = pytest.mark.gpu



def _specimen(n, seed, **kw):
    # The schedules of these tests (iterations at which the walls carry force, stop tests) were
    # written for dt = 0.5 sqrt(m_min / kn), the translational step without the rotational term of
    # assemblies.critical_dt; over a few hundred steps the instability that term prevents does
    # not develop.  Both engines of a comparison run the same spec.
    spec = assemblies.cubic_specimen(n, seed=seed, **kw)
    part = spec.kind == 0
    spec.params["dt"] = 0.5 * float(np.sqrt(np.min(spec.state[part, 33]) / np.max(spec.materials["Kn"])))
    return spec

def shared_state(cfg, n=150, seed=5, steps=250):
    spec = _specimen(n, seed=seed)
    o = OracleScene.from_spec(spec, threads=4)
    o.set_servo(cfg)
    o.step(steps)
    e = Engine(device=0)
    e.load(spec)
    e.put_body_state(o.bodies())
    e.put_interactions(o.interactions())
    e.put_scalars(o.scalars())
    e.set_servo(cfg)
    e.put_servo(o.servo_state())
    return spec, o, e


def compare_states(g, r, rtol):
    for k, name in enumerate(STATE_NAMES):
        a, b = g[k], r[k]
        if np.isinf(b) or np.isnan(b):
            assert np.isinf(a) == np.isinf(b) and np.isnan(a) == np.isnan(b), name
        else:
            assert a == pytest.approx(b, rel=rtol, abs=1e-300), name


@pytest.mark.parametrize("mode", ["consolidation", "shear"])
def test_one_controlled_step_matches_oracle(gpu, mode):
    if mode == "consolidation":
        cfg = servo_config(goalx=1e5, goaly=1e5, goalz=1e5, max_vel=1.0, iterate_num_max=7)
    else:
        cfg = servo_config(z_servo=0, shearMode=1, goalx=1e5, goaly=1e5, goalz=0.05, max_vel=1.0,
                           ramp_interval=40, ramp_chunks=4, iterate_num_max=7)
    spec, o, e = shared_state(cfg)
    for _ in range(9):   # crosses a gain update (every 7 steps) and, in shear, the end of the ramp
        o.step(1)
        e.step(1)
        e.sync()
        gb, rb = e.body_state(), o.bodies()
        assert np.allclose(gb[:6, 0:3], rb[:6, 0:3], rtol=1e-11, atol=1e-15)
        compare_states(e.servo_state(), o.servo_state(), rtol=1e-9)
        # continue both from the oracle's state so that only one step's differences count
        e.put_body_state(o.bodies())
        e.put_interactions(o.interactions())
        e.put_scalars(o.scalars())
        e.put_servo(o.servo_state())


def test_shop_reductions_match_oracle(gpu):
    cfg = servo_config(goalx=1e5, goaly=1e5, goalz=1e5, max_vel=1.0)
    spec, o, e = shared_state(cfg, steps=300)
    # the reductions read the forces of the last step: one step on both from the shared state
    o.step(1)
    e.step(1)
    e.sync()
    assert e.unbalanced_force() == pytest.approx(o.unbalanced_force(), rel=1e-9)
    assert e.unbalanced_force(True) == pytest.approx(o.unbalanced_force(True), rel=1e-9)
    sg, so = e.get_stress(2.5e-6), o.get_stress(2.5e-6)
    assert np.allclose(sg, so, rtol=1e-9, atol=1e-9 * np.abs(so).max())


def test_stop_at_iter_halts_and_resumes(gpu):
    cfg = servo_config(goalx=1e5, goaly=1e5, goalz=1e5, max_vel=1.0, solve_num_max=150,
                       f_threshold=1e9, fmin_threshold=1e9, unbf_tol=1e9)
    spec = _specimen(100, seed=4)
    e = Engine(device=0)
    e.load(spec)
    e.set_servo(cfg)
    e.step(400)
    e.sync()
    st = state_dict(e.servo_state())
    assert st["stopAtIter"] == 300            # as in the oracle (test_servo_oracle)
    assert e.scalars()[0] == 300
    b0 = e.body_state()
    assert np.all(b0[:, 7:13] == 0)            # the quiet step zeroed velocities
    e.step(5)
    e.sync()
    assert np.array_equal(e.body_state(), b0)  # halted: nothing moves
    s = e.servo_state().copy()
    s[STATE_NAMES.index("stopAtIter")] = -1
    e.put_servo(s)
    e.step(3)
    e.sync()
    assert e.scalars()[0] == 303


def test_quiet_flag(gpu):
    spec = _specimen(80, seed=2)
    e = Engine(device=0)
    e.load(spec)
    e.step(20)
    b0 = e.body_state()
    e.set_quiet(True)
    e.step(1)
    e.sync()
    b = e.body_state()
    assert np.all(b[:, 7:13] == 0)
    assert np.array_equal(b[:, 0:3], b0[:, 0:3])
    assert e.servo_state()[35] == 0


def test_graph_equals_eager_with_servo(gpu):
    cfg = servo_config(goalx=1e5, goaly=1e5, goalz=1e5, max_vel=1.0, iterate_num_max=10, solve_num_max=50,
                       echo_interval=25, savedata_interval=12)
    spec = _specimen(120, seed=9)
    a, b = Engine(device=0, use_graph=True), Engine(device=0, use_graph=False)
    for x in (a, b):
        x.load(spec)
        x.set_servo(cfg)
        x.step(120)
        x.sync()
    assert np.array_equal(a.body_state(), b.body_state())
    assert np.array_equal(a.servo_state(), b.servo_state(), equal_nan=True)
