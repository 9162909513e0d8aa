"""CompressionEngine, quiet flag and Shop reductions in the CPU oracle (no GPU).

The oracle restates CompressionEngine::action_cubic (pkg/dem/Compression.cpp:395-604, SOLE_GAIN
and NEW_SCHEME), NewtonIntegrator::quiet_system_flag (NewtonIntegrator.cpp:246-299),
Shop::unbalancedForce (Shop_01.cpp:148-188) and Shop::getStress (Shop_02.cpp:350-376); these
tests check each against its definition computed here from the oracle's own records.
"""
import math
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
from oracle import OracleScene  # noqa: E402
from sudodem_gb300 import assemblies  # noqa: E402
from sudodem_gb300.servo import servo_config, state_dict  # noqa: E402

# interaction record columns (include/sqdem.h)
ID1, ID2, REAL, KN, FN, FS, CD = 0, 1, 2, 23, slice(26, 29), slice(29, 32), slice(44, 47)


def specimen(n=120, seed=3, **kw):
    # These tests check the engine's bookkeeping (gains, clamps, iteration schedules) over a few
    # hundred steps whose schedules were written for dt = 0.5 sqrt(m_min / kn), the translational
    # step without the rotational term of critical_dt; over so few steps the rotational
    # instability that term prevents does not develop.
    spec = assemblies.cubic_specimen(n, seed=seed, **kw)
    part = spec.kind == 0
    spec.params["dt"] = 0.5 * float(np.sqrt(np.min(spec.state[part, 33]) / np.max(spec.materials["Kn"])))
    return spec, OracleScene.from_spec(spec, threads=2)


def test_first_run_gains_are_alpha_area_over_wall_stiffness():
    spec, o = specimen()
    # let particles reach the walls first (no engine), then add it
    o.set_servo(servo_config(goalx=1e5, goaly=1e5, goalz=1e5, max_vel=0.0))
    o.step(1)
    st = state_dict(o.servo_state())
    I = o.interactions()
    real = I[I[:, REAL] > 0]
    kn = np.zeros(6)
    for r in real:
        i = int(min(r[ID1], r[ID2]))
        if i < 6:
            kn[i] += r[KN]
    assert st["firstRun"] == 0
    box = spec.info["box"]
    x_area, y_area, z_area = box[1] * box[2], box[0] * box[2], box[1] * box[0]
    assert st["width0"] == box[0] and st["depth0"] == box[1] and st["height0"] == box[2]
    with np.errstate(divide="ignore"):
        want = [0.5 * x_area / kn[0], 0.5 * x_area / kn[1], 0.5 * y_area / kn[2], 0.5 * y_area / kn[3],
                0.5 * z_area / kn[4], 0.5 * z_area / kn[5]]
    got = [st["gain_x"], st["gain_x1"], st["gain_y"], st["gain_y1"], st["gain_z"], st["gain_z1"]]
    for g, w in zip(got, want):
        assert g == pytest.approx(w, rel=1e-12) or (math.isinf(g) and math.isinf(w))
    vols = [assemblies.shape_props(*spec.shape5[k])[0] for k in range(6, len(spec.kind))]
    assert st["particlesVolume"] == pytest.approx(sum(vols), rel=1e-14)


def test_consolidation_moves_walls_inward_toward_the_goal():
    spec, o = specimen(n=150, seed=5)
    o.set_servo(servo_config(goalx=1e5, goaly=1e5, goalz=1e5, max_vel=1.0, iterate_num_max=20))
    nsteps = 400
    o.step(nsteps)
    st = state_dict(o.servo_state())
    b = o.bodies()
    box = spec.info["box"]
    assert b[0, 0] > 0 and b[1, 0] < box[0] and b[4, 2] > 0 and b[5, 2] < box[2]
    assert st["width"] < box[0] and st["height"] < box[2]
    assert st["wsxx"] > 0 and st["wsyy"] > 0 and st["wszz"] > 0
    # each wall moved at most max_vel*dt per step
    assert b[0, 0] <= nsteps * 1.0 * spec.params["dt"] * (1 + 1e-12)


def test_wall_step_is_gain_times_stress_error_clamped():
    spec, o = specimen(n=150, seed=5)
    o.set_servo(servo_config(goalx=1e5, goaly=1e5, goalz=1e5, max_vel=0.05, iterate_num_max=1000))
    o.step(200)
    st0 = state_dict(o.servo_state())
    b0 = o.bodies()
    o.step(1)
    st = state_dict(o.servo_state())
    b = o.bodies()
    ms = 0.05 * spec.params["dt"]
    u = st["gain_x1"] * (st["wsxx_right"] - 1e5)
    want = math.copysign(min(abs(u), ms), u) if u != 0 else 0.0
    assert b[1, 0] - b0[1, 0] == pytest.approx(want, rel=1e-9, abs=1e-18)
    assert st["iterate_num"] == st0["iterate_num"] + 1


def test_shear_ramp_moves_top_and_bottom_by_ramp_velocity():
    spec, o = specimen(n=100, seed=7)
    cfg = servo_config(z_servo=0, shearMode=1, goalx=1e5, goaly=1e5, goalz=0.1, ramp_interval=100,
                       ramp_chunks=10, max_vel=0.0)
    o.set_servo(cfg)
    b0 = o.bodies()
    o.step(1)
    b = o.bodies()
    h = spec.info["box"][2]
    dt = spec.params["dt"]
    vel = float(np.float32(np.float32(1 / (50.0 / 10) + 1) / np.float32(10))) * 0.1 * 2.0
    assert b[4, 2] - b0[4, 2] == pytest.approx(vel * dt * h, rel=1e-12)
    assert b[5, 2] - b0[5, 2] == pytest.approx(-vel * dt * h, rel=1e-12)


def test_quiet_flag_zeroes_velocities_and_holds_positions():
    spec, o = specimen(n=80, seed=2)
    o.step(20)
    b0 = o.bodies()
    o.set_quiet(True)
    o.step(1)
    b = o.bodies()
    assert np.all(b[:, 7:13] == 0)
    assert np.array_equal(b[:, 0:3], b0[:, 0:3])
    assert o.servo_state()[35] == 0   # cleared by the step
    o.step(1)
    assert np.any(b[6:, 0:3] != o.bodies()[6:, 0:3]) or np.all(o.bodies()[6:, 16:19] == 0)


def test_unbalanced_force_and_stress_definitions():
    spec, o = specimen(n=150, seed=5)
    o.set_servo(servo_config(goalx=1e5, goaly=1e5, goalz=1e5, max_vel=1.0))
    o.step(300)
    b = o.bodies()
    I = o.interactions()
    real = I[I[:, REAL] > 0]
    g = np.array(spec.params["gravity"])
    dyn = np.arange(6, len(b))
    F = b[dyn, 16:19] + b[dyn, 33:34] * g
    num = np.sum(np.sqrt(F[:, 0] ** 2 + (F[:, 1] ** 2 + F[:, 2] ** 2)))
    fn, fs = real[:, FN], real[:, FS]
    nz = np.linalg.norm(fn, axis=1) != 0
    den = 2.0 * np.sum(np.linalg.norm(fn[nz] + fs[nz], axis=1))
    assert o.unbalanced_force() == pytest.approx(num / den, rel=1e-12)
    st = np.zeros((3, 3))
    for r in real:
        br = b[int(r[ID1]), 0:3] - b[int(r[ID2]), 0:3]
        st += np.outer(r[FN] + r[FS], br)
    vol = 2.5e-6
    assert np.allclose(o.get_stress(vol), st / vol, rtol=1e-12, atol=1e-9 * np.abs(st).max() / vol)


def test_stop_at_iter_when_consolidation_criteria_hold():
    spec, o = specimen(n=100, seed=4)
    o.set_servo(servo_config(goalx=1e5, goaly=1e5, goalz=1e5, max_vel=1.0, solve_num_max=150,
                             f_threshold=1e9, fmin_threshold=1e9, unbf_tol=1e9))
    o.step(400)
    st = state_dict(o.servo_state())
    # solve_num reaches 150 in the actions of iterations 149 and 299.  At 149 the walls carry no
    # force yet: mean stress 0, deviator/mean NaN, no stop (as in the reference).  At 299 the
    # test holds: O.run stops after that iteration, quiet requested.
    assert st["stopAtIter"] == 300
    assert o.scalars()[0] == 300
    b = o.bodies()
    assert np.all(b[:, 7:13] == 0)   # the quiet step zeroed velocities
