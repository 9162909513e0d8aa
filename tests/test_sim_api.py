"""The SudoDEM3D scripting surface (sudodem_gb300.sim): names, attributes, defaults and the
body/material packing handed to the C ABI.  No GPU needed except where marked."""
import math

import numpy as np
import pytest

from sudodem_gb300 import assemblies, sim


def build_example(O, n=8, seed=1):
    import random
    random.seed(seed)
    mat = sim.SuperquadricsMat(label="mat1", Kn=1e5, Ks=5e4, frictionAngle=math.atan(0.5), density=2650,
                               betan=0, betas=0)
    O.materials.append(mat)
    side = 10e-3
    O.bodies.append(sim.utils.wall(0, axis=0, sense=1, material=mat))
    O.bodies.append(sim.utils.wall(side, axis=0, sense=-1, material=mat))
    O.bodies.append(sim.utils.wall(0, axis=1, sense=1, material=mat))
    O.bodies.append(sim.utils.wall(side, axis=1, sense=-1, material=mat))
    O.bodies.append(sim.utils.wall(0, axis=2, sense=1, material=mat))
    O.bodies.append(sim.utils.wall(0.2, axis=2, sense=-1, material=mat))
    for k in range(n):
        b = sim.NewSuperquadrics2(1e-3, 0.9e-3, 0.8e-3, 0.7, 1.3, mat, True, False)
        b.state.pos = (2.5e-3 + 5e-3 * (k % 2), 2.5e-3 + 5e-3 * ((k // 2) % 2), 2e-3 + 2.6e-3 * (k // 4))
        O.bodies.append(b)
    O.engines = [sim.ForceResetter(),
                 sim.InsertionSortCollider([sim.Bo1_Superquadrics_Aabb(), sim.Bo1_Wall_Aabb()], verletDist=2e-4),
                 sim.InteractionLoop([sim.Ig2_Wall_Superquadrics_SuperquadricsGeom(),
                                      sim.Ig2_Superquadrics_Superquadrics_SuperquadricsGeom()],
                                     [sim.Ip2_SuperquadricsMat_SuperquadricsMat_SuperquadricsPhys()],
                                     [sim.SuperquadricsLaw()]),
                 sim.NewtonIntegrator(damping=0.3, gravity=(0, 0, -9.81), isSuperquadrics=1)]
    O.dt = 1e-6
    return mat


def test_reference_defaults():
    assert sim.NewtonIntegrator().damping == 0.2
    assert sim.NewtonIntegrator().exactAsphericalRot is True
    c = sim.InsertionSortCollider()
    assert (c.verletDist, c.targetInterv, c.minSweepDistFactor, c.sortAxis) == (-0.5, 50, 0.1, 0)
    m = sim.SuperquadricsMat()
    assert (m.Kn, m.Ks, m.frictionAngle, m.betan, m.betas) == (1e8, 1e5, 0.5, 0.0, 0.0)
    with pytest.raises(AttributeError):
        sim.NewtonIntegrator(nonexistent=1)


def test_aliases_map_to_superquadric_physics():
    assert issubclass(sim.Ip2_FrictMat_FrictMat_FrictPhys, sim.Ip2_SuperquadricsMat_SuperquadricsMat_SuperquadricsPhys)
    assert issubclass(sim.Law2_ScGeom_FrictPhys_CundallStrack, sim.SuperquadricsLaw)
    fm = sim.FrictMat(young=2e5, poisson=0.4, frictionAngle=0.3, density=2000)
    sm = fm.as_superquadrics()
    assert (sm.Kn, sm.Ks, sm.frictionAngle, sm.density) == (2e5, 0.4 * 2e5, 0.3, 2000)


def test_factory_matches_reference_body_setup():
    O = sim.Omega()
    sim.O.reset()
    mat = sim.SuperquadricsMat(density=2650)
    b = sim.NewSuperquadrics_rot2(1e-3, 0.8e-3, 0.9e-3, 0.6, 1.4, mat, 2.0, 0.0, 0.0, 0.0, False)
    props = b.shape._props()
    assert b.state.mass == 2650 * props[0]
    assert np.array_equal(b.state.inertia, props[1:4] * 2650)
    assert np.allclose(b.state.ori, [1, 0, 0, 0])
    assert b.aspherical
    w = sim.utils.wall(3.0, axis=2, sense=-1, material=mat)
    assert isinstance(w.shape, sim.Wall) and not w.dynamic and list(w.state.pos) == [0, 0, 3.0]
    del O


def test_engine_list_validation():
    O = sim.Omega()
    build_example(O)
    col, ilp, newton, runners = O._parse_engines()
    assert isinstance(col, sim.InsertionSortCollider) and newton.isSuperquadrics == 1
    O.engines = O.engines + [object()]
    with pytest.raises(NotImplementedError):
        O._parse_engines()


def test_packed_arrays_equal_assembly_spec_layout():
    O = sim.Omega()
    build_example(O, n=4)
    mats = O._material_table()
    assert len(mats) == 1
    kind, shape5, was, mat, sph, st, blocked = O._body_arrays()
    assert list(kind[:6]) == [1] * 6 and list(kind[6:]) == [0] * 4
    assert list(blocked[:6]) == [63] * 6 and list(blocked[6:]) == [0] * 4
    assert np.all(np.isnan(st[:, 28:31]))
    assert np.allclose(np.linalg.norm(st[6:, 3:7], axis=1), 1.0)


@pytest.mark.gpu
def test_script_runs_on_gpu_and_matches_engine(gpu):
    O = sim.Omega()
    build_example(O, n=8)
    O.run(200, True)
    z = np.array([b.state.pos[2] for b in O.bodies][6:])
    assert np.all(np.isfinite(z)) and O.iter == 200
    # same scene straight through the C ABI
    kind, shape5, was, mat, sph, st, blocked = O._body_arrays()
    O2 = sim.Omega()
    build_example(O2, n=8)
    m = O2._material_table()[0]
    kind2, shape52, was2, mat2, sph2, st2, _ = O2._body_arrays()
    from sudodem_gb300 import Engine
    e = Engine(device=0)
    e.set_materials([m.Kn], [m.Ks], [m.frictionAngle], [m.betan], [m.betas], [m.density])
    e.set_params(dt=1e-6, gravity=(0, 0, -9.81), damping=0.3, verletDist=2e-4)
    e.set_bodies(kind2, shape52, was2, mat2, sph2, st2)
    e.step(200)
    e.sync()
    assert np.array_equal(e.body_state()[:, 0:3], np.array([b.state.pos for b in O.bodies]))


def build_consolidation(O, n=27, seed=2):
    """example2_consol.py-style specimen: six walls first (left, right, front, back, bottom, top),
    particles inside, CompressionEngine between InteractionLoop and NewtonIntegrator."""
    import random
    random.seed(seed)
    mat = sim.SuperquadricsMat(label="mat1", Kn=1e5, Ks=5e4, frictionAngle=math.atan(0.3), density=2650)
    wmat = sim.SuperquadricsMat(label="wallmat", Kn=1e5, Ks=0.0, frictionAngle=0.0)
    O.materials.append(mat)
    O.materials.append(wmat)
    side = 6e-3
    for pos, ax, se in ((0, 0, 1), (side, 0, -1), (0, 1, 1), (side, 1, -1), (0, 2, 1), (side, 2, -1)):
        O.bodies.append(sim.utils.wall(pos, axis=ax, sense=se, material=wmat))
    for k in range(n):
        b = sim.NewSuperquadrics2(1e-3, 0.9e-3, 0.8e-3, 1.2, 1.2, mat, True, False)
        b.state.pos = (1.2e-3 + 1.8e-3 * (k % 3), 1.2e-3 + 1.8e-3 * ((k // 3) % 3), 1.2e-3 + 1.8e-3 * (k // 9))
        O.bodies.append(b)
    triax = sim.CompressionEngine(goalx=1e5, goaly=1e5, goalz=1e5, max_vel=1.0, gain_alpha=0.5,
                                  iterate_num_max=20, echo_interval=50)
    newton = sim.NewtonIntegrator(damping=0.3, gravity=(0, 0, 0), isSuperquadrics=1)
    O.engines = [sim.ForceResetter(),
                 sim.InsertionSortCollider([sim.Bo1_Superquadrics_Aabb(), sim.Bo1_Wall_Aabb()], verletDist=1e-4),
                 sim.InteractionLoop([sim.Ig2_Wall_Superquadrics_SuperquadricsGeom(),
                                      sim.Ig2_Superquadrics_Superquadrics_SuperquadricsGeom()],
                                     [sim.Ip2_SuperquadricsMat_SuperquadricsMat_SuperquadricsPhys()],
                                     [sim.SuperquadricsLaw()]),
                 triax, newton]
    O.dt = 2e-6
    return triax, newton


def test_compression_engine_attributes_and_placement():
    ce = sim.CompressionEngine()
    # reference defaults (Compression.hpp:160-215)
    assert (ce.goalx, ce.max_vel, ce.gain_alpha, ce.iterate_num_max, ce.solve_num_max) == (0, 1, 0.5, 100, 2000)
    assert (ce.savedata_interval, ce.ramp_interval, ce.ramp_chunks, ce.unbf_tol) == (12, 10000, 400, 0.01)
    with pytest.raises(AttributeError):
        sim.CompressionEngine(goal_x=1)
    from sudodem_gb300.servo import CONFIG_NAMES
    cfg = sim.CompressionEngine(goalx=2e5, z_servo=False, top_wall_activated=False)._config()
    assert cfg[CONFIG_NAMES.index("goalx")] == 2e5 and cfg[CONFIG_NAMES.index("z_servo")] == 0
    assert cfg[CONFIG_NAMES.index("top_wall_activated")] == 0 and cfg[0] == 1
    O = sim.Omega()
    triax, newton = build_consolidation(O)
    O._parse_engines()
    assert O._servo is triax
    O.engines = O.engines[:3] + [newton, triax]     # after Newton: not the reference's order
    with pytest.raises(NotImplementedError):
        O._parse_engines()


@pytest.mark.gpu
def test_consolidation_script_matches_engine(gpu):
    O = sim.O          # utils functions act on the global scene, as in the reference
    O.reset()
    triax, newton = build_consolidation(O)
    O.run(300, True)
    assert triax.width < 6e-3 and triax.height < 6e-3   # walls moved in
    pos = np.array([b.state.pos for b in O.bodies])
    # the same through the C ABI
    O2 = sim.Omega()
    t2, n2 = build_consolidation(O2)
    mats = O2._material_table()
    kind, shape5, was, mat, sph, st, _ = O2._body_arrays()
    from sudodem_gb300 import Engine
    e = Engine(device=0)
    e.set_materials([m.Kn for m in mats], [m.Ks for m in mats], [m.frictionAngle for m in mats],
                    [m.betan for m in mats], [m.betas for m in mats], [m.density for m in mats])
    e.set_params(dt=2e-6, gravity=(0, 0, 0), damping=0.3, verletDist=1e-4)
    e.set_bodies(kind, shape5, was, mat, sph, st)
    e.set_servo(t2._config())
    e.step(300)
    e.sync()
    assert np.array_equal(e.body_state()[:, 0:3], pos)
    # quiet flag through NewtonIntegrator, Shop functions through utils
    newton.quiet_system_flag = True
    O.run(1, True)
    assert np.all(np.array([b.state.vel for b in O.bodies]) == 0)
    assert not newton.quiet_system_flag
    assert np.isfinite(sim.utils.unbalancedForce())
    assert sim.utils.getStress(1e-6).shape == (3, 3)
    mean, dev = triax.getStress()
    assert np.isfinite(mean) and np.isfinite(dev)
    O.reset()


def use_hertz_mindlin(O, G=2e8, nu=0.3):
    """Switch an example scene to the Hertz-Mindlin functor set and SuperquadricsMat2."""
    m = O.materials[0]
    m2 = sim.SuperquadricsMat2(label=m.label, Kn=m.Kn, Ks=m.Ks, frictionAngle=m.frictionAngle, density=m.density,
                               G=G, nu=nu)
    O.materials[0] = m2
    for b in O.bodies:
        b.mat = m2
    ilp = O.engines[2]
    ilp.geomDispatcher = [sim.Ig2_Wall_Superquadrics_SuperquadricsGeom2(),
                          sim.Ig2_Superquadrics_Superquadrics_SuperquadricsGeom2()]
    ilp.physDispatcher = [sim.Ip2_SuperquadricsMat2_SuperquadricsMat2_HertzMindlinPhys()]
    ilp.lawDispatcher = [sim.SuperquadricsLaw2()]
    return m2


def test_hertz_mindlin_functor_set():
    assert sim.SuperquadricsMat2().G == 29e9 and sim.SuperquadricsMat2().nu == 0.15   # Superquadrics.hpp:270-271
    O = sim.Omega()
    build_example(O, n=4)
    O._parse_engines()
    assert O._contactModel == "linear"
    use_hertz_mindlin(O)
    O._parse_engines()
    assert O._contactModel == "hertz_mindlin"
    O.engines[2].lawDispatcher = [sim.SuperquadricsLaw()]
    with pytest.raises(NotImplementedError):
        O._parse_engines()


@pytest.mark.gpu
def test_hertz_mindlin_script_matches_engine(gpu):
    O = sim.Omega()
    build_example(O, n=8)
    m2 = use_hertz_mindlin(O)
    O.run(300, True)
    assert O._engine.contact_model() == "hertz_mindlin"
    O2 = sim.Omega()
    build_example(O2, n=8)
    m = O2._material_table()[0]
    kind, shape5, was, mat, sph, st, _ = O2._body_arrays()
    from sudodem_gb300 import Engine
    e = Engine(device=0)
    e.set_materials([m.Kn], [m.Ks], [m.frictionAngle], [m.betan], [m.betas], [m.density])
    e.set_material_moduli([m2.G], [m2.nu])
    e.set_contact_model("hertz_mindlin")
    e.set_params(dt=1e-6, gravity=(0, 0, -9.81), damping=0.3, verletDist=2e-4)
    e.set_bodies(kind, shape5, was, mat, sph, st)
    e.step(300)
    e.sync()
    assert np.array_equal(e.body_state()[:, 0:3], np.array([b.state.pos for b in O.bodies]))
