"""Snapshot / restore (sqdem_snapshot, sqdem_restore; O.save / O.load of the scripting surface):
a context restored from a snapshot continues bit for bit as the original would."""
import numpy as np
import pytest

from sudodem_gb300 import Engine, SqdemError, assemblies, sim
from sudodem_gb300.servo import servo_config

pytestmark = pytest.mark.gpu


def same(a, b):
    assert np.array_equal(a.body_state(), b.body_state())
    assert np.array_equal(a.interactions(True), b.interactions(True))
    assert np.array_equal(a.scalars(), b.scalars())
    assert np.array_equal(a.servo_state(), b.servo_state(), equal_nan=True)


@pytest.mark.parametrize("case", ["walled_servo", "periodic", "mixed"])
def test_restored_context_continues_bitwise(gpu, case):
    if case == "periodic":
        spec = assemblies.periodic_cell(300, seed=3, solid_fraction=0.35, strain_rate=2.0)
        prec = "fp64"
    else:
        spec = assemblies.cubic_specimen(150, seed=6)
        prec = "mixed" if case == "mixed" else "fp64"
    a = Engine(precision=prec)
    a.load(spec)
    if case != "periodic":
        a.set_servo(servo_config(goalx=1e5, goaly=1e5, goalz=1e5, max_vel=1.0, iterate_num_max=9,
                                 echo_interval=7, savedata_interval=5))
    a.step(40)
    a.sync()
    blob = a.snapshot()
    a.step(35)
    a.sync()
    b = Engine(precision=prec, contacts_per_body=24)   # another capacity: the table still fits
    b.restore(blob)
    b.step(35)
    b.sync()
    same(a, b)
    if case == "periodic":
        assert np.array_equal(a.cell(), b.cell())


def test_restore_refuses_foreign_bytes(gpu):
    e = Engine()
    with pytest.raises(SqdemError):
        e.restore(b"not a snapshot" * 10)


def test_save_load_script_continues_bitwise(gpu, tmp_path):
    from test_sim_api import build_consolidation
    O = sim.Omega()
    build_consolidation(O)
    O.run(60, True)
    f = str(tmp_path / "scene.sqdem")
    O.save(f)
    O.run(40, True)
    pos = np.array([b.state.pos for b in O.bodies])
    O2 = sim.Omega()
    O2.load(f)
    assert O2.iter == 60 and len(O2.bodies) == len(O.bodies)
    O2.run(40, True)
    assert np.array_equal(np.array([b.state.pos for b in O2.bodies]), pos)
