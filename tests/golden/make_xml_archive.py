"""Writes tests/golden/sq_scene.xml.bz2: a SudoDEM3D scene archive as O.save would write it
for a small superquadric scene (a wall, two superquadrics, one contact with history, one shared
material), composed by hand from the reference's serialization macros.  It is the fixture the
archive reader is checked against and that the writer must reproduce byte for byte.

Every element, in order, restates a declaration of the reference:
  Scene                core/Scene.hpp:97-127         Body          core/Body.hpp:83-97
  BodyContainer        core/BodyContainer.hpp:73      State         core/State.hpp:53-64
  InteractionContainer core/InteractionContainer.hpp:121 (filled by preSave, .cpp:143-150)
  Shape                core/Shape.hpp:26-29          Wall          pkg/common/Wall.hpp:11-13
  Superquadrics        pkg/dem/Superquadrics.hpp:138-146
  Bound / Aabb         core/Bound.hpp:24-31 (min, max noSave) / pkg/common/Aabb.hpp:24
  Material             core/Material.hpp:38-41       SuperquadricsMat pkg/dem/Superquadrics.hpp:247-264
  Interaction          core/Interaction.hpp:50-59 (iterLastSeen, linIx noSave)
  SuperquadricsGeom    pkg/dem/Superquadrics.hpp:182-196
  SuperquadricsPhys    pkg/dem/Superquadrics.hpp:300-309 -> FrictPhys pkg/dem/FrictPhys.hpp:19-20
                       -> NormShearPhys / NormPhys pkg/common/NormShearPhys.hpp:10-25
  NodeContainer / FEContainer pkg/fem/Node.hpp:185 / pkg/fem/FEContainer.hpp:122
  EnergyTracker        core/EnergyTracker.hpp:54-57 (accumulator: lib/base/openmp-accu.hpp:205)
  Cell                 core/Cell.hpp:143-156
  Eigen types          lib/base/Math.hpp:653-743
Each class body starts with its base class (lib/serialization/Serializable.hpp:121-131).

The class ids and object ids are written out by hand below, in the order Boost assigns them:
a class takes the next id when first met, as a pointer's static type (silently) or as an
object; object ids count tracked objects (every Serializable, base-class parts included).
Run: python tests/golden/make_xml_archive.py
"""
import bz2
import os

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "sq_scene.xml.bz2")

lines = []
depth = [0]


def R(x):
    return format(float(x), ".17e")


def start(name, attrs=""):
    lines.append(("\n" + "\t" * depth[0] if depth[0] else "") + "<" + name + (" " + attrs if attrs else "") + ">")
    depth[0] += 1


def end(name, compound=True):
    depth[0] -= 1
    lines.append(("\n" + "\t" * depth[0] if compound else "") + "</" + name + ">")


def leaf(name, text, attrs=""):
    lines.append("\n" + "\t" * depth[0] + "<" + name + (" " + attrs if attrs else "") + ">" + text + "</" + name + ">")


def empty(name, attrs):
    lines.append("\n" + "\t" * depth[0] + "<" + name + " " + attrs + "></" + name + ">")


def vec(name, comps, vals, attrs="", ints=False):
    start(name, attrs)
    for c, v in zip(comps, vals):
        leaf(c, str(int(v)) if ints else R(v))
    end(name)


def v3(name, v, attrs=""):
    vec(name, "xyz", v, attrs)


def quat(name, q, attrs=""):
    vec(name, "wxyz", q, attrs)


I3 = (1.0, 0, 0, 0, 1.0, 0, 0, 0, 1.0)


def mat3(name, m, attrs=""):
    vec(name, ["m%d%d" % (i, j) for i in range(3) for j in range(3)], m, attrs)


# the scene's values
DT, ITER, TIME = 2.5e-6, 120, 3.0e-4
MAT = dict(density=2650.0, Kn=1.0e5, Ks=5.0e4, frictionAngle=0.4636476090008061, betan=0.0, betas=0.0, strength=100.0)
B1 = dict(r=(1.0e-3, 1.2e-3, 0.9e-3), eps=(0.6, 1.4), pos=(1.0e-3, 2.0e-3, 1.05e-3),
          ori=(0.9238795325112867, 0.0, 0.3826834323650898, 0.0), vel=(1.0e-3, -2.0e-3, 5.0e-4),
          angVel=(0.5, -0.25, 0.125), angMom=(1.0e-12, 2.0e-12, -3.0e-12), mass=1.1e-5,
          inertia=(4.1e-12, 3.9e-12, 4.4e-12), bref=(0.99e-3, 2.01e-3, 1.04e-3), sweep=1.5e-5, lui=117,
          color=(0.25, 0.5, 0.75))
B2 = dict(r=(1.1e-3, 0.95e-3, 1.05e-3), eps=(1.2, 0.8), pos=(2.8e-3, 2.1e-3, 1.1e-3),
          ori=(0.8660254037844387, 0.5, 0.0, 0.0), vel=(-1.0e-3, 0.0, 2.5e-4), angVel=(0.0, 0.75, -0.5),
          angMom=(0.0, 3.0e-12, -2.0e-12), mass=1.2e-5, inertia=(4.3e-12, 4.6e-12, 4.0e-12),
          bref=(2.81e-3, 2.1e-3, 1.1e-3), sweep=1.25e-5, lui=118, color=(0.5, 0.125, 0.0625))
GEOM = dict(PenetrationDepth=2.5e-6, contactAngle=(0.7, -0.3), contactPoint=(1.9e-3, 2.05e-3, 1.07e-3),
            shearInc=(1.0e-9, -2.0e-9, 5.0e-10), relativeVn=(-1.0e-3, 1.0e-4, 0.0),
            relativeVs=(2.0e-4, -1.0e-4, 3.0e-5), normal=(0.98, 0.05, 0.1916), twist_axis=(0.0, 0.0, 1.0e-6),
            point1=(1.91e-3, 2.06e-3, 1.08e-3), point2=(1.89e-3, 2.04e-3, 1.06e-3),
            orthonormal_axis=(0.0, 1.0e-7, 0.0))
PHYS = dict(kn=1.0e5, normalForce=(-0.245, -0.0125, -0.0479), ks=5.0e4, shearForce=(1.0e-3, -2.0e-3, 3.0e-4),
            tan=0.5)

Z3 = (0.0, 0.0, 0.0)
lines.append('<?xml version="1.0" encoding="UTF-8" standalone="yes" ?>\n<!DOCTYPE boost_serialization>\n'
             '<boost_serialization signature="serialization::archive" version="12">\n')
# class ids: 0 shared_ptr<Scene>, 1 Scene, 2 Serializable
start("scene", 'class_id="0" tracking_level="0" version="1"')
start("px", 'class_id="1" tracking_level="1" version="0" object_id="_0"')
empty("Serializable", 'class_id="2" tracking_level="1" version="0" object_id="_1"')
leaf("dt", R(DT)); leaf("iter", str(ITER)); leaf("subStepping", "0"); leaf("subStep", "-1")
leaf("time", R(TIME)); leaf("speed", R(0)); leaf("stopAtIter", "0"); leaf("stopAtTime", R(0))
leaf("isPeriodic", "0"); leaf("trackEnergy", "0"); leaf("doSort", "0"); leaf("runInternalConsistencyChecks", "1")
leaf("selectedBody", "-1"); leaf("flags", "0")
# 3 list<string>
start("tags", 'class_id="3" tracking_level="0" version="0"')
leaf("count", "1"); leaf("item_version", "0"); leaf("item", "author=fixture~(sudodem_gb300)")
end("tags")
# 4 vector<shared_ptr<Engine>> (Engine is not registered: no element is written)
start("engines", 'class_id="4" tracking_level="0" version="0"'); leaf("count", "0"); leaf("item_version", "1"); end("engines")
start("_nextEngines"); leaf("count", "0"); leaf("item_version", "1"); end("_nextEngines")
# 5 shared_ptr<BodyContainer>, 6 BodyContainer, 7 vector<shared_ptr<Body>>, 8 shared_ptr<Body>, 9 Body
start("bodies", 'class_id="5" tracking_level="0" version="1"')
start("px", 'class_id="6" tracking_level="1" version="0" object_id="_2"')
empty("Serializable", 'object_id="_3"')
start("body", 'class_id="7" tracking_level="0" version="0"')
leaf("count", "3"); leaf("item_version", "1")


def state(oid, s, first):
    # 13 shared_ptr<State>, 14 State, 15 Se3r, 16 Vector3r, 17 Quaternionr
    start("state", 'class_id="13" tracking_level="0" version="1"' if first else "")
    start("px", ('class_id="14" tracking_level="1" version="0" ' if first else 'class_id_reference="14" ')
          + 'object_id="_%d"' % oid)
    empty("Serializable", 'object_id="_%d"' % (oid + 1))
    start("se3", 'class_id="15" tracking_level="0" version="0"' if first else "")
    v3("position", s["pos"], 'class_id="16" tracking_level="0" version="0"' if first else "")
    quat("orientation", s["ori"], 'class_id="17" tracking_level="0" version="0"' if first else "")
    end("se3")
    v3("vel", s["vel"]); leaf("mass", R(s["mass"])); v3("angVel", s["angVel"]); v3("angMom", s["angMom"])
    v3("inertia", s["inertia"]); v3("refPos", s["refPos"]); quat("refOri", (1.0, 0, 0, 0))
    leaf("blockedDOFs", str(s["dofs"])); leaf("isDamped", "1"); leaf("densityScaling", R(1.0))
    end("px")
    end("state")


def bound(oid, lui, ref, sweep, first):
    # 21 shared_ptr<Bound>, 22 Bound (static type), 23 Aabb
    start("bound", 'class_id="21" tracking_level="0" version="1"' if first else "")
    start("px", ('class_id="23" class_name="Aabb" tracking_level="1" version="0" ' if first else
                 'class_id_reference="23" ') + 'object_id="_%d"' % oid)
    start("Bound", ('class_id="22" tracking_level="1" version="0" ' if first else "") + 'object_id="_%d"' % (oid + 1))
    empty("Serializable", 'object_id="_%d"' % (oid + 2))
    leaf("lastUpdateIter", str(lui)); v3("refPos", ref); leaf("sweepLength", R(sweep)); v3("color", (1.0, 1.0, 1.0))
    end("Bound")
    end("px")
    end("bound")


def shape_base(oid, color, first):
    start("Shape", ('class_id="19" tracking_level="1" version="0" ' if first else "") + 'object_id="_%d"' % oid)
    empty("Serializable", 'object_id="_%d"' % (oid + 1))
    v3("color", color); leaf("wire", "0"); leaf("highlight", "0")
    end("Shape")


# body 0: the wall (ids _4.._16)
start("item", 'class_id="8" tracking_level="0" version="1"')
start("px", 'class_id="9" tracking_level="1" version="0" object_id="_4"')
empty("Serializable", 'object_id="_5"')
leaf("id", "0"); leaf("groupMask", "1"); leaf("flags", "1")
# 10 shared_ptr<Material>, 11 Material (static type), 12 SuperquadricsMat
start("material", 'class_id="10" tracking_level="0" version="1"')
start("px", 'class_id="12" class_name="SuperquadricsMat" tracking_level="1" version="0" object_id="_6"')
start("Material", 'class_id="11" tracking_level="1" version="0" object_id="_7"')
empty("Serializable", 'object_id="_8"')
leaf("id", "0"); leaf("label", "grains"); leaf("density", R(MAT["density"]))
end("Material")
for k in ("Kn", "Ks", "frictionAngle", "betan", "betas"):
    leaf(k, R(MAT[k]))
leaf("IsSplitable", "0"); leaf("strength", R(MAT["strength"]))
end("px")
end("material")
state(9, dict(pos=Z3, ori=(1.0, 0, 0, 0), vel=Z3, mass=0.0, angVel=Z3, angMom=Z3, inertia=Z3, refPos=Z3, dofs=63),
      True)
# 18 shared_ptr<Shape>, 19 Shape (static type), 20 Wall
start("shape", 'class_id="18" tracking_level="0" version="1"')
start("px", 'class_id="20" class_name="Wall" tracking_level="1" version="0" object_id="_11"')
shape_base(12, (1.0, 1.0, 1.0), True)
leaf("sense", "1"); leaf("axis", "2")
end("px")
end("shape")
bound(14, 117, Z3, 0.0, True)
# 24 map<int,shared_ptr<Interaction>>: empty for the wall (the pair class is not registered yet)
start("intrs", 'class_id="24" tracking_level="0" version="0"'); leaf("count", "0"); leaf("item_version", "0"); end("intrs")
leaf("clumpId", "-1"); leaf("chain", "-1"); leaf("iterBorn", "0"); leaf("timeBorn", R(0))
end("px")
end("item")


def sq_body(bid, b, oid, other, intr_first):
    start("item")
    start("px", 'class_id_reference="9" object_id="_%d"' % oid)
    empty("Serializable", 'object_id="_%d"' % (oid + 1))
    leaf("id", str(bid)); leaf("groupMask", "1"); leaf("flags", "3")
    start("material"); empty("px", 'class_id_reference="12" object_id_reference="_6"'); end("material")
    state(oid + 2, dict(pos=b["pos"], ori=b["ori"], vel=b["vel"], mass=b["mass"], angVel=b["angVel"],
                        angMom=b["angMom"], inertia=b["inertia"], refPos=Z3, dofs=0), False)
    start("shape")
    # 25 Superquadrics (first time), then class_id_reference
    start("px", ('class_id="25" class_name="Superquadrics" tracking_level="1" version="0" ' if bid == 1 else
                 'class_id_reference="25" ') + 'object_id="_%d"' % (oid + 4))
    shape_base(oid + 5, b["color"], False)
    v3("rxyz", b["r"])
    for k, v in zip(("rx", "ry", "rz", "eps1", "eps2"), (*b["r"], *b["eps"])):
        leaf(k, R(v))
    leaf("isSphere", "0")
    # 26 Vector2r
    vec("eps", "xy", b["eps"], 'class_id="26" tracking_level="0" version="0"' if bid == 1 else "")
    end("px")
    end("shape")
    bound(oid + 7, b["lui"], b["bref"], b["sweep"], False)
    start("intrs")
    leaf("count", "1"); leaf("item_version", "0")
    # 27 pair<const int, shared_ptr<Interaction>>, 28 shared_ptr<Interaction>, 29 Interaction
    start("item", 'class_id="27" tracking_level="0" version="0"' if intr_first else "")
    leaf("first", str(other))
    start("second", 'class_id="28" tracking_level="0" version="1"' if intr_first else "")
    if intr_first:
        interaction(oid + 10)
    else:
        empty("px", 'class_id_reference="29" object_id_reference="_27"')
    end("second")
    end("item")
    end("intrs")
    leaf("clumpId", "-1"); leaf("chain", "-1"); leaf("iterBorn", "0"); leaf("timeBorn", R(0))
    end("px")
    end("item")


def interaction(oid):
    # object ids: _27 Interaction, _28 Serializable, _29.._31 geom, _32.._37 phys
    start("px", 'class_id="29" tracking_level="1" version="0" object_id="_%d"' % oid)
    empty("Serializable", 'object_id="_%d"' % (oid + 1))
    leaf("id1", "1"); leaf("id2", "2"); leaf("iterMadeReal", "100")
    # 30 shared_ptr<IGeom>, 31 IGeom (static type), 32 SuperquadricsGeom
    start("geom", 'class_id="30" tracking_level="0" version="1"')
    start("px", 'class_id="32" class_name="SuperquadricsGeom" tracking_level="1" version="0" object_id="_%d"' % (oid + 2))
    start("IGeom", 'class_id="31" tracking_level="1" version="0" object_id="_%d"' % (oid + 3))
    empty("Serializable", 'object_id="_%d"' % (oid + 4))
    end("IGeom")
    g = GEOM
    leaf("PenetrationDepth", R(g["PenetrationDepth"]))
    vec("contactAngle", "xy", g["contactAngle"])
    for k in ("contactPoint", "shearInc", "relativeVn", "relativeVs", "normal", "twist_axis", "point1", "point2"):
        v3(k, g[k])
    v3("point11", Z3); v3("point22", Z3)
    leaf("isShearNew", "0")
    v3("orthonormal_axis", g["orthonormal_axis"])
    end("px")
    end("geom")
    # 33 shared_ptr<IPhys>, 34 IPhys (static type), 35 SuperquadricsPhys, 36 FrictPhys, 37 NormShearPhys,
    # 38 NormPhys
    start("phys", 'class_id="33" tracking_level="0" version="1"')
    start("px", 'class_id="35" class_name="SuperquadricsPhys" tracking_level="1" version="0" object_id="_%d"' % (oid + 5))
    start("FrictPhys", 'class_id="36" tracking_level="1" version="0" object_id="_%d"' % (oid + 6))
    start("NormShearPhys", 'class_id="37" tracking_level="1" version="0" object_id="_%d"' % (oid + 7))
    start("NormPhys", 'class_id="38" tracking_level="1" version="0" object_id="_%d"' % (oid + 8))
    start("IPhys", 'class_id="34" tracking_level="1" version="0" object_id="_%d"' % (oid + 9))
    empty("Serializable", 'object_id="_%d"' % (oid + 10))
    end("IPhys")
    leaf("kn", R(PHYS["kn"])); v3("normalForce", PHYS["normalForce"])
    end("NormPhys")
    leaf("ks", R(PHYS["ks"])); v3("shearForce", PHYS["shearForce"])
    end("NormShearPhys")
    leaf("tangensOfFrictionAngle", R(PHYS["tan"]))
    end("FrictPhys")
    v3("normalViscous", Z3); v3("shearViscous", Z3); leaf("betan", R(0)); leaf("betas", R(0))
    end("px")
    end("phys")
    # 39 Vector3i
    vec("cellDist", "xyz", (0, 0, 0), 'class_id="39" tracking_level="0" version="0"', ints=True)
    leaf("iterBorn", "100")
    end("px")


# body 1: _17.._26, its interaction _27.._37 (written in full in body 1's intrs)
sq_body(1, B1, 17, 2, True)
# body 2: _38.._47; its intrs refers to the interaction written above
sq_body(2, B2, 38, 1, False)
end("body")
end("px")
end("bodies")
# 40 shared_ptr<NodeContainer>, 41 NodeContainer, 42 vector<shared_ptr<Node>>
start("nodes", 'class_id="40" tracking_level="0" version="1"')
start("px", 'class_id="41" tracking_level="1" version="0" object_id="_48"')
empty("Serializable", 'object_id="_49"')
start("node", 'class_id="42" tracking_level="0" version="0"'); leaf("count", "0"); leaf("item_version", "1"); end("node")
end("px"); end("nodes")
# 43 shared_ptr<FEContainer>, 44 FEContainer, 45 vector<shared_ptr<Element>>
start("elements", 'class_id="43" tracking_level="0" version="1"')
start("px", 'class_id="44" tracking_level="1" version="0" object_id="_50"')
empty("Serializable", 'object_id="_51"')
start("element", 'class_id="45" tracking_level="0" version="0"'); leaf("count", "0"); leaf("item_version", "1")
end("element")
end("px"); end("elements")
# 46 shared_ptr<InteractionContainer>, 47 InteractionContainer, 48 vector<shared_ptr<Interaction>>
start("interactions", 'class_id="46" tracking_level="0" version="1"')
start("px", 'class_id="47" tracking_level="1" version="0" object_id="_52"')
empty("Serializable", 'object_id="_53"')
start("interaction", 'class_id="48" tracking_level="0" version="0"'); leaf("count", "1"); leaf("item_version", "1")
start("item"); empty("px", 'class_id_reference="29" object_id_reference="_27"'); end("item")
end("interaction")
leaf("serializeSorted", "0"); leaf("dirty", "0")
end("px"); end("interactions")
# 49 shared_ptr<EnergyTracker>, 50 EnergyTracker, 51 OpenMPArrayAccumulator<Real>, 52 map<string,int>,
# 53 vector<bool>
start("energy", 'class_id="49" tracking_level="0" version="1"')
start("px", 'class_id="50" tracking_level="1" version="0" object_id="_54"')
empty("Serializable", 'object_id="_55"')
start("energies", 'class_id="51" tracking_level="0" version="0"'); leaf("size", "0"); end("energies")
start("names", 'class_id="52" tracking_level="0" version="0"'); leaf("count", "0"); leaf("item_version", "0"); end("names")
start("resetStep", 'class_id="53" tracking_level="0" version="0"'); leaf("count", "0"); end("resetStep")
end("px"); end("energy")
# 54 vector<shared_ptr<Material>>: the shared material, written in body 0
start("materials", 'class_id="54" tracking_level="0" version="0"'); leaf("count", "1"); leaf("item_version", "1")
start("item"); empty("px", 'class_id_reference="12" object_id_reference="_6"'); end("item")
end("materials")
# the scene's bound: a null shared_ptr<Bound>
start("bound"); lines.append("\n" + "\t" * depth[0] + '<px class_id="-1"></px>'); end("bound")
# 55 shared_ptr<Cell>, 56 Cell, 57 Matrix3r
start("cell", 'class_id="55" tracking_level="0" version="1"')
start("px", 'class_id="56" tracking_level="1" version="0" object_id="_56"')
empty("Serializable", 'object_id="_57"')
mat3("trsf", I3, 'class_id="57" tracking_level="0" version="0"')
for k in ("refHSize", "hSize", "prevHSize"):
    mat3(k, I3)
for k in ("velGrad", "nextVelGrad", "prevVelGrad"):
    mat3(k, (0,) * 9)
leaf("homoDeform", "1"); leaf("velGradChanged", "0")
end("px"); end("cell")
# 58 vector<shared_ptr<Serializable>>, 59 vector<shared_ptr<DisplayParameters>>
start("miscParams", 'class_id="58" tracking_level="0" version="0"'); leaf("count", "0"); leaf("item_version", "1")
end("miscParams")
start("dispParams", 'class_id="59" tracking_level="0" version="0"'); leaf("count", "0"); leaf("item_version", "1")
end("dispParams")
end("px")
end("scene")
lines.append("\n</boost_serialization>\n")

TEXT = "".join(lines)

if __name__ == "__main__":
    text = TEXT
    with bz2.open(OUT, "wb") as f:
        f.write(text.encode("utf-8"))
    print(OUT, len(text), "characters")
