"""Batches of specimens: one graph launch steps every scene; each scene's results are those of
its context stepped alone (bitwise), in both precision forms, with the CompressionEngine."""
import ctypes as C

import numpy as np
import pytest

from sudodem_gb300 import Batch, Engine, SqdemError, assemblies
from sudodem_gb300.servo import servo_config

pytestmark = pytest.mark.gpu

SERVO = servo_config(z_servo=0, shearMode=1, goalx=1e5, goaly=1e5, goalz=0.05, max_vel=1.0,
                     ramp_interval=30, ramp_chunks=3, iterate_num_max=10)


def specs(k=4, seed=11):
    sizes = [60, 150, 90, 220, 40, 130][:k]
    return [assemblies.cubic_specimen(n, seed=seed + i, friction=0.2 + 0.1 * i) for i, n in enumerate(sizes)]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_scenes_equal_independent_runs(gpu, precision):
    ss = specs()
    b = Batch(len(ss), precision=precision)
    b.load(ss, servo=SERVO)
    b.scenes[2].set_servo(servo_config(enabled=0))   # one scene without the engine
    b.step(25)
    b.sync()
    for i, spec in enumerate(ss):
        e = Engine(precision=precision)
        e.load(spec)
        if i != 2:
            e.set_servo(SERVO)
        e.step(25)
        e.sync()
        assert np.array_equal(b.scenes[i].body_state(), e.body_state()), i
        assert np.array_equal(b.scenes[i].interactions(True), e.interactions(True)), i
        assert np.array_equal(b.scenes[i].servo_state(), e.servo_state(), equal_nan=True), i
    b.close()


def test_batch_graph_rebuilt_after_a_scene_changes(gpu):
    ss = specs(3, seed=21)
    b = Batch(3)
    b.load(ss)
    b.step(10)
    b.scenes[1].set_servo(SERVO)   # the step's kernel sequence of scene 1 changes
    b.step(10)
    b.sync()
    e = Engine()
    e.load(ss[1])
    e.step(10)
    e.set_servo(SERVO)
    e.step(10)
    e.sync()
    assert np.array_equal(b.scenes[1].body_state(), e.body_state())
    assert b.launch_count() > 0
    b.close()


def test_batch_sync_reports_a_scene_overflow(gpu):
    ss = specs(2, seed=31)
    b = Batch(2, contacts_per_body=1)
    b.load(ss)
    b.step(3)
    with pytest.raises(SqdemError) as ei:
        b.sync()
    assert ei.value.status == 3
    b.close()


def test_batch_time_e2e_round_trips_kinematics(gpu):
    ss = specs(3, seed=41)
    b = Batch(3)
    b.load(ss, servo=SERVO)
    b.step(2)
    b.sync()
    kin = np.concatenate([e.kinematics() for e in b.scenes])
    a, c = kin.copy(), np.zeros_like(kin)
    ms = b.time_e2e(2, a.ctypes.data, c.ctypes.data)     # in -> out -> in
    assert ms > 0
    b.sync()
    now = np.concatenate([e.kinematics() for e in b.scenes])
    assert np.array_equal(a, now)
    # the same two steps from the same state on independent contexts
    ref = []
    for i, spec in enumerate(ss):
        e = Engine()
        e.load(spec)
        e.set_servo(SERVO)
        e.step(4)
        e.sync()
        ref.append(e.kinematics())
    assert np.array_equal(now, np.concatenate(ref))
    b.close()
