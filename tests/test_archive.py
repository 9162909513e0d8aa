"""SudoDEM3D scene archives (O.save / O.load, .xml / .xml.bz2 / .xml.gz): sudodem_gb300.archive.

CPU: the reader against the hand-composed fixture tests/golden/sq_scene.xml.bz2 (every value,
and the writer reproducing it byte for byte); round trips of a real dense state (the oracle's
bodies and contact history) through the three file kinds, bit for bit in every field the
archive carries; and a continuation test: a state written to an archive and read back steps
bit for bit like the original state stepped with the reference's load semantics (collider
re-initialised, the bounds' min/max recomputed: they are not saved, core/Bound.hpp:30-31).
GPU: the same continuation with the engine: export, re-import, step, compare bit for bit.
"""
import os
import sys

import numpy as np
import pytest

from oracle import OracleScene
from parity_util import by_pair
from sudodem_gb300 import archive, assemblies

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "golden", "sq_scene.xml.bz2")
TILE = os.path.join(HERE, "golden", "config1_tile.npz")
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_xml_archive as FX  # noqa: E402


class OracleAsEngine:
    """The oracle behind the engine calls archive.from_engine makes."""

    def __init__(self, orc, model="linear"):
        self.o, self.model = orc, model

    def body_state(self):
        return self.o.bodies()

    def interactions(self, include_potential=True):
        return self.o.interactions()

    def scalars(self):
        return self.o.scalars()

    def contact_model(self):
        return self.model

    def cell(self):
        return self.o.cell()


def test_fixture_values():
    a = archive.load(FIXTURE)
    assert (a.dt, a.iter, a.time) == (FX.DT, FX.ITER, FX.TIME)
    assert not a.isPeriodic and a.tags == ["author=fixture~(sudodem_gb300)"]
    assert a.n == 3 and list(a.kind) == [1, 0, 0] and list(a.mat) == [0, 0, 0]
    assert tuple(a.wall[0]) == (2, 1)
    m = a.materials[0]
    assert m["cls"] == "SuperquadricsMat" and m["label"] == "grains"
    for k in ("density", "Kn", "Ks", "frictionAngle", "betan", "betas", "strength"):
        assert m[k] == FX.MAT[k]
    for i, B in ((1, FX.B1), (2, FX.B2)):
        assert tuple(a.shape5[i]) == (*B["r"], *B["eps"])
        st = a.state[i]
        assert tuple(st[0:3]) == B["pos"] and tuple(st[3:7]) == B["ori"] and tuple(st[7:10]) == B["vel"]
        assert tuple(st[10:13]) == B["angVel"] and tuple(st[13:16]) == B["angMom"]
        assert st[33] == B["mass"] and tuple(st[34:37]) == B["inertia"]
        assert tuple(st[28:31]) == B["bref"] and st[31] == B["sweep"] and st[32] == B["lui"]
        assert np.all(np.isnan(st[22:28]))      # min / max are not saved
        assert tuple(a.shapeColor[i]) == B["color"] and a.flags[i] == 3 and a.blockedDOFs[i] == 0
    assert a.blockedDOFs[0] == 63 and a.flags[0] == 1 and a.state[0, 32] == 117
    assert a.intr.shape == (1, 57)
    r = a.intr[0]
    g, p = FX.GEOM, FX.PHYS
    assert tuple(r[0:4]) == (1, 2, 1, 1)
    assert r[4] == g["PenetrationDepth"] and tuple(r[5:7]) == g["contactAngle"]
    assert tuple(r[7:10]) == g["contactPoint"] and tuple(r[10:13]) == g["normal"] and tuple(r[13:16]) == g["shearInc"]
    assert tuple(r[16:19]) == g["point1"] and tuple(r[19:22]) == g["point2"] and r[22] == 0
    assert (r[23], r[24], r[25]) == (p["kn"], p["ks"], p["tan"])
    assert tuple(r[26:29]) == p["normalForce"] and tuple(r[29:32]) == p["shearForce"]
    assert tuple(r[32:35]) == g["twist_axis"] and tuple(r[35:38]) == g["orthonormal_axis"]
    assert tuple(r[38:41]) == g["relativeVn"] and tuple(r[41:44]) == g["relativeVs"]
    assert a.iterMadeReal[0] == 100 and a.iterBorn_i[0] == 100


def test_writer_reproduces_fixture_byte_for_byte():
    a = archive.load(FIXTURE)
    assert archive.dumps(archive.scene_graph(a)) == FX.TEXT


def _carried(a):
    """The fields an archive carries, for comparison: min/max of the bounds are not saved, the
    bound history of bodies without a bound, the physics of interactions without physics and the
    Hertz-Mindlin geometry of linear contacts do not exist in the reference's objects."""
    st = a.state.copy()
    st[:, 16:28] = np.nan
    st[~a.hasBound, 28:33] = 0
    st[~a.hasBound, 28:31] = np.nan
    r = a.intr.copy()
    r[r[:, 2] == 0, 23:32] = 0
    r[~a.hm, 47:57] = 0
    return st, r


def _dense_walled_oracle(steps=6, threads=None):
    spec = assemblies.walled_lattice(400, seed=5, box=14e-3, per_side=5, spacing=2.1e-3)
    o = OracleScene.from_spec(spec, threads=threads or os.cpu_count())
    o.step(steps)
    return spec, o


@pytest.mark.parametrize("suffix", [".xml", ".xml.bz2", ".xml.gz"])
def test_round_trip_dense_state(tmp_path, suffix):
    spec, o = _dense_walled_oracle()
    a = archive.from_engine(OracleAsEngine(o), spec, tags=["author=test"])
    assert np.sum(a.intr[:, 2] != 0) > 300
    path = str(tmp_path / ("scene" + suffix))
    archive.save(path, a)
    b = archive.load(path)
    sa, ra = _carried(a)
    sb, rb = _carried(b)
    assert np.array_equal(sa, sb, equal_nan=True)
    assert np.array_equal(ra, rb, equal_nan=True)
    for k in ("kind", "shape5", "isSphere", "wall", "mat", "hasBound", "blockedDOFs", "isDamped", "refPos", "refOri",
              "groupMask", "flags", "iterMadeReal", "iterBorn_i", "betas2", "viscous"):
        assert np.array_equal(getattr(a, k), getattr(b, k)), k
    assert (b.dt, b.iter, b.time, b.materials, b.tags) == (a.dt, a.iter, a.time, a.materials, a.tags)
    # writing what was read gives the same file content
    assert archive.dumps(archive.scene_graph(b)) == archive.dumps(archive.scene_graph(a))


def _oracle_from_archive(a, params, threads=1):
    spec = archive.spec_from_archive(a, params)
    o = OracleScene.from_spec(spec, threads=threads)
    st = a.state.copy()
    st[:, 22:28] = np.nan
    o.set_bodies(st)
    o.set_interactions(a.intr)
    s = o.scalars()
    s[0] = a.iter
    s[8] = 0
    o.set_scalars(s)
    return o


def test_oracle_continues_bit_for_bit_through_an_archive(tmp_path):
    """Write the oracle's state to an archive, read it into a new oracle, and step both: the
    original, reset to the reference's load semantics (fresh collider state, bounds' min/max
    unset, the interactions without geometry or physics dropped: InteractionContainer::preSave
    keeps only the others, core/InteractionContainer.cpp:143-150), and the one read back must
    agree bit for bit after 40 steps.  (Per-body force sums follow the interaction order and the
    thread that adds them, as the reference's do: both keep the saved order and run on one
    thread.)"""
    spec, o = _dense_walled_oracle(steps=8, threads=1)
    a = archive.from_engine(OracleAsEngine(o), spec)
    path = str(tmp_path / "s.xml.bz2")
    archive.save(path, a)
    b = _oracle_from_archive(archive.load(path), spec.params)
    st = o.bodies()
    st[:, 22:28] = np.nan
    o.set_bodies(st)
    recs = o.interactions()
    o.set_interactions(recs[(recs[:, 2] != 0) | (recs[:, 3] != 0)])
    o.set_scalars(b.scalars())
    o.step(40)
    b.step(40)
    assert np.array_equal(o.bodies(), b.bodies(), equal_nan=True)
    ro, rb = by_pair(o.interactions()), by_pair(b.interactions())
    real = [k for k, r in ro.items() if r[2] != 0 or r[3] != 0]
    assert len(real) > 300 and all(np.array_equal(ro[k], rb[k]) for k in real)


def test_reader_maps_the_engines_of_an_archive():
    """An archive the reference writes carries O.engines; the reader describes each engine
    (class and attributes) for the scripting layer.  Here: a hand-written engine list."""
    a = archive.load(FIXTURE)
    assert a.engines == []


@pytest.mark.gpu
def test_engine_continues_bit_for_bit_through_an_archive(gpu, tmp_path):
    from sudodem_gb300 import Engine
    spec = assemblies.walled_lattice(400, seed=5, box=14e-3, per_side=5, spacing=2.1e-3)
    A = Engine(device=0)
    A.load(spec)
    A.step(8)
    A.sync()
    a = archive.from_engine(A, spec)
    path = str(tmp_path / "s.xml.bz2")
    archive.save(path, a)
    B, _ = archive.to_engine(archive.load(path), params=spec.params, device=0)
    # B holds A's state in every carried field
    sb, rb = _carried(archive.from_engine(B, spec))
    sa, ra = _carried(a)
    assert np.array_equal(sa, sb, equal_nan=True)
    assert np.array_equal(ra[np.lexsort((ra[:, 1], ra[:, 0]))], rb[np.lexsort((rb[:, 1], rb[:, 0]))], equal_nan=True)
    st = A.body_state()
    st[:, 22:28] = np.nan
    A.put_body_state(st)
    recs = A.interactions(True)
    A.put_interactions(recs[(recs[:, 2] != 0) | (recs[:, 3] != 0)])
    A.put_scalars(B.scalars())
    A.step(40)
    B.step(40)
    A.sync()
    B.sync()
    assert np.array_equal(A.body_state()[:, 0:16], B.body_state()[:, 0:16])
    GA, GB = by_pair(A.interactions(True)), by_pair(B.interactions(True))
    real = [k for k, r in GA.items() if r[2] != 0]
    assert len(real) > 300 and all(np.array_equal(GA[k], GB[k]) for k in real)


ENGINES = """<engines class_id="4" tracking_level="0" version="0">
			<count>3</count>
			<item_version>1</item_version>
			<item class_id="100" tracking_level="0" version="1">
				<px class_id="101" class_name="ForceResetter" tracking_level="1" version="0" object_id="_1000">
					<Engine class_id="102" tracking_level="1" version="0" object_id="_1001">
						<Serializable object_id="_1002"></Serializable>
						<dead>0</dead>
						<ompThreads>-1</ompThreads>
						<label></label>
					</Engine>
				</px>
			</item>
			<item>
				<px class_id="103" class_name="InsertionSortCollider" tracking_level="1" version="0" object_id="_1003">
					<verletDist>2.00000000000000004e-04</verletDist>
					<targetInterv>30</targetInterv>
					<boundDispatcher class_id="104" tracking_level="0" version="1">
						<px class_id="105" tracking_level="1" version="0" object_id="_1004">
							<functors class_id="106" tracking_level="0" version="0">
								<count>1</count>
								<item_version>1</item_version>
								<item class_id="107" tracking_level="0" version="1">
									<px class_id="108" class_name="Bo1_Superquadrics_Aabb" tracking_level="1" version="0" object_id="_1005"></px>
								</item>
							</functors>
						</px>
					</boundDispatcher>
				</px>
			</item>
			<item>
				<px class_id="109" class_name="NewtonIntegrator" tracking_level="1" version="0" object_id="_1006">
					<damping>3.00000000000000004e-01</damping>
					<gravity class_id="16" tracking_level="0" version="0">
						<x>0.00000000000000000e+00</x>
						<y>0.00000000000000000e+00</y>
						<z>-9.81000000000000050e+00</z>
					</gravity>
					<isSuperquadrics>1</isSuperquadrics>
				</px>
			</item>
		</engines>"""


def test_reader_maps_engines_and_the_scripting_layer_loads_the_fixture(tmp_path):
    """O.load of an archive: bodies, materials, time and the engines the GPU path knows (here a
    hand-written engine list in the reference's layout, with attributes left out that the
    reader does not need)."""
    from sudodem_gb300 import sim
    import bz2
    text = FX.TEXT
    i0 = text.index('<engines class_id="4"')
    i1 = text.index("</engines>") + len("</engines>")
    path = str(tmp_path / "e.xml.bz2")
    with bz2.open(path, "wb") as f:
        f.write((text[:i0] + ENGINES + text[i1:]).encode())
    a = archive.load(path)
    assert [e[0] for e in a.engines] == ["ForceResetter", "InsertionSortCollider", "NewtonIntegrator"]
    O = sim.Omega()
    O.load(path)
    assert len(O.bodies._b) == 3 and O.dt == FX.DT and O.iter == FX.ITER and O.time == FX.TIME
    assert isinstance(O.bodies._b[0].shape, sim.Wall) and isinstance(O.bodies._b[1].shape, sim.Superquadrics)
    assert O.materials[0].label == "grains" and O.materials[0].Kn == FX.MAT["Kn"]
    b1 = O.bodies._b[1]
    assert tuple(b1.state.pos) == FX.B1["pos"] and tuple(b1.state.angVel) == FX.B1["angVel"]
    kinds = [type(e).__name__ for e in O.engines]
    assert kinds == ["ForceResetter", "InsertionSortCollider", "NewtonIntegrator"]
    col, newton = O.engines[1], O.engines[2]
    assert col.verletDist == 2e-4 and col.targetInterv == 30
    assert [type(f).__name__ for f in col.boundFunctors] == ["Bo1_Superquadrics_Aabb"]
    assert newton.damping == 0.3 and newton.gravity == (0.0, 0.0, -9.81) and newton.isSuperquadrics == 1
    assert O.loadSkipped == []
    assert O._pendingArchive is not None


@pytest.mark.gpu
def test_omega_save_load_archive_continues(gpu, tmp_path):
    """The scripting layer: O.save to .xml.bz2 and O.load back give the same state, and the run
    continues from it."""
    from sudodem_gb300 import sim
    O = sim.Omega()
    mat = sim.SuperquadricsMat(Kn=1e5, Ks=5e4, frictionAngle=0.5, density=2650)
    mat.label = "grains"
    O.materials.append(mat)
    O.bodies.append(sim.utils.wall(0, axis=2, sense=1, material=mat))
    for k in range(40):
        b = sim.NewSuperquadrics2(1e-3, 1.1e-3, 0.9e-3, 0.7 + 0.02 * k, 1.2, mat, True, False)
        b.state.pos = (2.1e-3 * (k % 5), 2.1e-3 * ((k // 5) % 4), 1.2e-3 + 2.05e-3 * (k // 20))
        O.bodies.append(b)
    O.engines = [sim.ForceResetter(),
                 sim.InsertionSortCollider([sim.Bo1_Superquadrics_Aabb(), sim.Bo1_Wall_Aabb()], verletDist=2e-4),
                 sim.InteractionLoop([sim.Ig2_Wall_Superquadrics_SuperquadricsGeom(),
                                      sim.Ig2_Superquadrics_Superquadrics_SuperquadricsGeom()],
                                     [sim.Ip2_SuperquadricsMat_SuperquadricsMat_SuperquadricsPhys()],
                                     [sim.SuperquadricsLaw()]),
                 sim.NewtonIntegrator(damping=0.3, gravity=(0, 0, -9.81), isSuperquadrics=1)]
    O.dt = 2e-6
    O.run(300, True)
    path = str(tmp_path / "o.xml.bz2")
    O.save(path)
    before = [b.state.pos.copy() for b in O.bodies._b]
    O2 = sim.Omega()
    O2.load(path)
    O2.engines = O.engines
    assert O2.iter == O.iter and O2.materials[0].label == "grains"
    assert all(np.array_equal(p, b.state.pos) for p, b in zip(before, O2.bodies._b))
    O2.run(50, True)
    assert O2.iter == O.iter + 50
    assert len(O2.interactions) > 0
