"""SudoDEM3D scene archives (``O.save`` / ``O.load`` with ``.xml``, ``.xml.bz2``, ``.xml.gz``).

The reference saves the whole Scene with Boost.Serialization's XML archive, compressed by the
file name's suffix (lib/serialization/ObjectIO.hpp:28-64, core/Omega.cpp:230-279).  This module
reads and writes that format for the superquadric path: the bodies (Superquadrics and Wall
shapes, State, Aabb bound, shared SuperquadricsMat / SuperquadricsMat2 materials) and the
interactions with their history (SuperquadricsGeom / SuperquadricsGeom2 and SuperquadricsPhys /
SuperquadricsHertzMindlinPhys), the periodic Cell, dt, iter and time.  It needs no Boost: the
archive layout is restated from the reference's serialization macros and Boost's XML archive
rules, below.

Layout of one class (lib/serialization/Serializable.hpp:121-131, _REGISTER_BOOST_ATTRIBUTES):
the base class as an element named after it, then every attribute of the class's
SUDODEM_CLASS_* declaration in declaration order, except those flagged Attr::noSave.  The
attribute lists written here are those of the declarations cited in ``_CLASSES``.  Eigen types
are written component by component (lib/base/Math.hpp:653-743); boost::shared_ptr as a ``px``
pointer element (class version 1, untracked); std containers as ``count``, ``item_version``
and ``item`` elements; std::vector<bool> without ``item_version``.

Boost's bookkeeping, restated: a class gets the next class id when the archive first meets it,
either as the static type of a pointer (registered silently) or as an object; its first
appearance carries ``class_id``, ``tracking_level`` and ``version`` (and ``class_name`` when a
pointer's dynamic type is met for the first time and differs from the static type), later
pointers to it carry ``class_id_reference``.  Every object of a class serialized through
pointers (all Serializable classes) is tracked: the next ``object_id`` on its first appearance,
``object_id_reference`` on a pointer to an object already written.  Base-class objects are
tracked objects of their own.  Doubles are written with 17 digits after the point in
scientific notation (max_digits10), so a value read back is the value written, bit for bit.

What is written follows what the reference would write for the same scene, with these
limits, each stated where it applies: the engine list is written empty (the script sets
O.engines after O.load; the reader maps the engines of an archive written by the reference),
colours are white unless given (``body_extra``), and each body's ``intrs`` map holds the saved
(real) interactions only, which is what the reference rebuilds from on load
(core/InteractionContainer.cpp:143-167: only interactions with geom or phys are kept).
"""
import bz2
import gzip
import io
import math
import xml.etree.ElementTree as ET

import numpy as np

from .shapes import BODY_STRIDE, INTR_STRIDE

ARCHIVE_VERSION = 12          # Boost.Serialization library version written in the header
ID_NONE = -1                  # Body::ID_NONE (core/Body.cpp:8)
FLAG_BOUNDED, FLAG_ASPHERICAL = 1, 2   # core/Body.hpp:36
DOF_ALL = 63                  # State::DOF_ALL (core/State.hpp:21-23)


def _open(path, mode):
    if path.endswith(".bz2"):
        return bz2.open(path, mode)
    if path.endswith(".gz"):
        return gzip.open(path, mode)
    return open(path, mode)


def is_xml_filename(path):
    """ObjectIO::isXmlFilename (lib/serialization/ObjectIO.hpp:28-30)."""
    return path.endswith(".xml") or path.endswith(".xml.bz2") or path.endswith(".xml.gz")


# ------------------------------------------------------------------------------------------
# Text of primitives (boost/archive/basic_text_oprimitive, xml_oarchive)
def _fmt_real(x):
    x = float(x)
    if math.isnan(x):
        return "-nan" if math.copysign(1.0, x) < 0 else "nan"
    if math.isinf(x):
        return "inf" if x > 0 else "-inf"
    return format(x, ".17e")


def _parse_real(t):
    t = t.strip()
    low = t.lower()
    if low in ("nan", "-nan", "+nan"):
        return -math.nan if low.startswith("-") else math.nan
    return float(t)


def _esc(s):
    return (s.replace("&", "&amp;").replace("<", "&lt;").replace(">", "&gt;").replace("'", "&apos;")
            .replace('"', "&quot;"))


# ------------------------------------------------------------------------------------------
# Writer: Boost's xml_oarchive start/end/preamble and class/object bookkeeping
class _Writer:
    def __init__(self):
        self.buf = []
        self.depth = 0
        self.pending = False
        self.indent_next = False
        self.classes = {}     # key -> [class_id, initialized]
        self.objects = {}     # id(python object) -> object_id
        self.nobj = 0
        self.keep = []        # keeps written objects alive so their id() stays unique

    # basic_xml_oarchive::save_start / end_preamble / save_end
    def start(self, name):
        self.end_preamble()
        if self.depth > 0:
            self.buf.append("\n" + "\t" * self.depth)
        self.depth += 1
        self.buf.append("<" + name)
        self.pending = True
        self.indent_next = False

    def attr(self, k, v):
        self.buf.append(' %s="%s"' % (k, v))

    def end_preamble(self):
        if self.pending:
            self.buf.append(">")
            self.pending = False

    def end(self, name):
        self.end_preamble()
        self.depth -= 1
        if self.indent_next:
            self.buf.append("\n" + "\t" * self.depth)
        self.indent_next = True
        self.buf.append("</%s>" % name)
        if self.depth == 0:
            self.buf.append("\n")

    def register(self, key):
        c = self.classes.get(key)
        if c is None:
            c = [len(self.classes), False]
            self.classes[key] = c
            return c, True
        return c, False

    # primitives
    def prim(self, name, text):
        self.start(name)
        self.end_preamble()
        self.buf.append(text)
        self.end(name)

    def real(self, name, x):
        self.prim(name, _fmt_real(x))

    def int(self, name, i):
        self.prim(name, str(int(i)))

    def bool(self, name, b):
        self.prim(name, "1" if b else "0")

    def string(self, name, s):
        self.prim(name, _esc(s))

    # an object of a class with class information (save_object)
    def obj(self, name, key, tracked, version, body):
        self.start(name)
        c, _ = self.register(key)
        if not c[1]:
            self.attr("class_id", c[0])
            self.attr("tracking_level", 1 if tracked else 0)
            self.attr("version", version)
            c[1] = True
        if tracked:
            self.attr("object_id", "_%d" % self.nobj)
            self.nobj += 1
        self.end_preamble()
        body()
        self.end(name)

    # Eigen types (lib/base/Math.hpp:653-743): untracked classes, version 0
    def vec(self, name, key, comps, values):
        def body():
            for c, v in zip(comps, values):
                if key.endswith("i"):
                    self.int(c, v)
                else:
                    self.real(c, v)
        self.obj(name, key, False, 0, body)

    def v2(self, name, v):
        self.vec(name, "Vector2r", ("x", "y"), v)

    def v3(self, name, v):
        self.vec(name, "Vector3r", ("x", "y", "z"), v)

    def v3i(self, name, v):
        self.vec(name, "Vector3i", ("x", "y", "z"), v)

    def quat(self, name, q):
        self.vec(name, "Quaternionr", ("w", "x", "y", "z"), q)

    def mat3(self, name, m):
        m = np.asarray(m, dtype=np.float64).reshape(3, 3)
        self.vec(name, "Matrix3r", tuple("m%d%d" % (i, j) for i in range(3) for j in range(3)), m.reshape(9))

    def se3(self, name, pos, ori):
        def body():
            self.v3("position", pos)
            self.quat("orientation", ori)
        self.obj(name, "Se3r", False, 0, body)

    # boost::shared_ptr<T>: the wrapper (untracked, version 1) holding the pointer "px"
    def sptr(self, name, static, o):
        self.obj(name, "shared_ptr<%s>" % static, False, 1, lambda: self.ptr("px", static, o))

    def ptr(self, name, static, o):
        self.start(name)
        self.register(static)
        if o is None:
            self.attr("class_id", -1)
            self.end_preamble()
            self.end(name)
            return
        c, new = self.register(o.cls)
        if not c[1]:
            self.attr("class_id", c[0])
            if new:
                self.attr("class_name", o.cls)
            self.attr("tracking_level", 1)
            self.attr("version", 0)
            c[1] = True
        else:
            self.attr("class_id_reference", c[0])
        oid = self.objects.get(id(o))
        if oid is not None:
            self.attr("object_id_reference", "_%d" % oid)
            self.end_preamble()
            self.end(name)
            return
        self.objects[id(o)] = self.nobj
        self.keep.append(o)
        self.attr("object_id", "_%d" % self.nobj)
        self.nobj += 1
        self.end_preamble()
        _CLASSES[o.cls](self, o)
        self.end(name)

    # std containers (boost/serialization/collections_save_imp.hpp, vector.hpp, map.hpp)
    def seq(self, name, key, items, item_version, write_item):
        def body():
            self.int("count", len(items))
            if item_version is not None:
                self.int("item_version", item_version)
            for it in items:
                write_item("item", it)
        self.obj(name, key, False, 0, body)

    def ptr_vector(self, name, static, items):
        self.seq(name, "vector<shared_ptr<%s>>" % static, items, 1, lambda n, o: self.sptr(n, static, o))

    def text(self):
        head = ('<?xml version="1.0" encoding="UTF-8" standalone="yes" ?>\n<!DOCTYPE boost_serialization>\n'
                '<boost_serialization signature="serialization::archive" version="%d">\n' % ARCHIVE_VERSION)
        return head + "".join(self.buf) + "</boost_serialization>\n"


class SObj:
    """A Serializable instance: its class name (the archive's class_name) and attributes."""

    def __init__(self, cls, **fields):
        self.cls = cls
        self.f = fields

    def __getitem__(self, k):
        return self.f[k]

    def get(self, k, default=None):
        return self.f.get(k, default)


# ------------------------------------------------------------------------------------------
# Class bodies: base object, then attributes in declaration order
def _base(w, base, o):
    w.obj(base, base, True, 0, lambda: _CLASSES[base](w, o))


def _serializable(w, o):
    pass   # lib/serialization/Serializable.hpp:245: no attributes


def _scene(w, o):
    # core/Scene.hpp:97-127
    _base(w, "Serializable", o)
    w.real("dt", o["dt"])
    w.int("iter", o["iter"])
    w.bool("subStepping", False)
    w.int("subStep", -1)
    w.real("time", o["time"])
    w.real("speed", 0.0)
    w.int("stopAtIter", 0)
    w.real("stopAtTime", 0.0)
    w.bool("isPeriodic", o["isPeriodic"])
    w.bool("trackEnergy", False)
    w.bool("doSort", False)
    w.bool("runInternalConsistencyChecks", True)
    w.int("selectedBody", -1)
    w.int("flags", 0)
    w.seq("tags", "list<string>", o["tags"], 0, lambda n, s: w.string(n, s))
    w.ptr_vector("engines", "Engine", [])
    w.ptr_vector("_nextEngines", "Engine", [])
    w.sptr("bodies", "BodyContainer", o["bodies"])
    w.sptr("nodes", "NodeContainer", SObj("NodeContainer"))
    w.sptr("elements", "FEContainer", SObj("FEContainer"))
    w.sptr("interactions", "InteractionContainer", o["interactions"])
    w.sptr("energy", "EnergyTracker", SObj("EnergyTracker"))
    w.ptr_vector("materials", "Material", o["materials"])
    w.sptr("bound", "Bound", None)
    w.sptr("cell", "Cell", o["cell"])
    w.ptr_vector("miscParams", "Serializable", [])
    w.ptr_vector("dispParams", "DisplayParameters", [])


def _body_container(w, o):
    # core/BodyContainer.hpp:73
    _base(w, "Serializable", o)
    w.ptr_vector("body", "Body", o["body"])


def _node_container(w, o):
    _base(w, "Serializable", o)          # pkg/fem/Node.hpp:185
    w.ptr_vector("node", "Node", [])


def _fe_container(w, o):
    _base(w, "Serializable", o)          # pkg/fem/FEContainer.hpp:122
    w.ptr_vector("element", "Element", [])


def _energy_tracker(w, o):
    # core/EnergyTracker.hpp:54-57; OpenMPArrayAccumulator as size + item<i> (lib/base/openmp-accu.hpp:205)
    _base(w, "Serializable", o)
    w.obj("energies", "OpenMPArrayAccumulator<Real>", False, 0, lambda: w.int("size", 0))
    w.seq("names", "map<string,int>", [], 0, None)
    w.seq("resetStep", "vector<bool>", [], None, None)


def _body(w, o):
    # core/Body.hpp:83-97 (no SPH / liquid-migration fields: off in the reference's build)
    _base(w, "Serializable", o)
    w.int("id", o["id"])
    w.int("groupMask", o["groupMask"])
    w.int("flags", o["flags"])
    w.sptr("material", "Material", o["material"])
    w.sptr("state", "State", o["state"])
    w.sptr("shape", "Shape", o["shape"])
    w.sptr("bound", "Bound", o["bound"])

    def pair(name, kv):
        def body():
            w.int("first", kv[0])
            w.sptr("second", "Interaction", kv[1])
        w.obj(name, "pair<int,shared_ptr<Interaction>>", False, 0, body)
    w.seq("intrs", "map<int,shared_ptr<Interaction>>", o["intrs"], 0, pair)
    w.int("clumpId", o["clumpId"])
    w.int("chain", o["chain"])
    w.int("iterBorn", o["iterBorn"])
    w.real("timeBorn", o["timeBorn"])


def _state(w, o):
    # core/State.hpp:53-64
    _base(w, "Serializable", o)
    w.se3("se3", o["pos"], o["ori"])
    w.v3("vel", o["vel"])
    w.real("mass", o["mass"])
    w.v3("angVel", o["angVel"])
    w.v3("angMom", o["angMom"])
    w.v3("inertia", o["inertia"])
    w.v3("refPos", o["refPos"])
    w.quat("refOri", o["refOri"])
    w.int("blockedDOFs", o["blockedDOFs"])
    w.bool("isDamped", o["isDamped"])
    w.real("densityScaling", o["densityScaling"])


def _shape(w, o):
    # core/Shape.hpp:26-29
    _base(w, "Serializable", o)
    w.v3("color", o.get("color", (1.0, 1.0, 1.0)))
    w.bool("wire", o.get("wire", False))
    w.bool("highlight", o.get("highlight", False))


def _superquadrics(w, o):
    # pkg/dem/Superquadrics.hpp:138-146
    _base(w, "Shape", o)
    w.v3("rxyz", (o["rx"], o["ry"], o["rz"]))
    w.real("rx", o["rx"])
    w.real("ry", o["ry"])
    w.real("rz", o["rz"])
    w.real("eps1", o["eps1"])
    w.real("eps2", o["eps2"])
    w.bool("isSphere", o["isSphere"])
    w.v2("eps", (o["eps1"], o["eps2"]))


def _wall(w, o):
    # pkg/common/Wall.hpp:11-13
    _base(w, "Shape", o)
    w.int("sense", o["sense"])
    w.int("axis", o["axis"])


def _bound(w, o):
    # core/Bound.hpp:24-31 (min and max are noSave)
    _base(w, "Serializable", o)
    w.int("lastUpdateIter", o["lastUpdateIter"])
    w.v3("refPos", o["refPos"])
    w.real("sweepLength", o["sweepLength"])
    w.v3("color", o.get("color", (1.0, 1.0, 1.0)))


def _aabb(w, o):
    _base(w, "Bound", o)                 # pkg/common/Aabb.hpp:24: no attributes


def _material(w, o):
    # core/Material.hpp:38-41
    _base(w, "Serializable", o)
    w.int("id", o["id"])
    w.string("label", o.get("label", ""))
    w.real("density", o["density"])


def _sq_mat(w, o):
    # pkg/dem/Superquadrics.hpp:247-264
    _base(w, "Material", o)
    for k in ("Kn", "Ks", "frictionAngle", "betan", "betas"):
        w.real(k, o[k])
    w.bool("IsSplitable", o.get("IsSplitable", False))
    w.real("strength", o.get("strength", 100.0))


def _sq_mat2(w, o):
    # pkg/dem/Superquadrics.hpp:266-277
    _base(w, "SuperquadricsMat", o)
    w.real("G", o["G"])
    w.real("nu", o["nu"])


def _interaction(w, o):
    # core/Interaction.hpp:50-59 (iterLastSeen and linIx are noSave)
    _base(w, "Serializable", o)
    w.int("id1", o["id1"])
    w.int("id2", o["id2"])
    w.int("iterMadeReal", o["iterMadeReal"])
    w.sptr("geom", "IGeom", o["geom"])
    w.sptr("phys", "IPhys", o["phys"])
    w.v3i("cellDist", o["cellDist"])
    w.int("iterBorn", o["iterBorn"])


def _igeom(w, o):
    _base(w, "Serializable", o)          # core/IGeom.hpp:18: no attributes


def _iphys(w, o):
    _base(w, "Serializable", o)          # core/IPhys.hpp:18: no attributes


def _sq_geom(w, o):
    # pkg/dem/Superquadrics.hpp:182-196
    _base(w, "IGeom", o)
    w.real("PenetrationDepth", o["PenetrationDepth"])
    w.v2("contactAngle", o["contactAngle"])
    for k in ("contactPoint", "shearInc", "relativeVn", "relativeVs", "normal", "twist_axis", "point1", "point2",
              "point11", "point22"):
        w.v3(k, o[k])
    w.bool("isShearNew", o["isShearNew"])
    w.v3("orthonormal_axis", o["orthonormal_axis"])


def _sq_geom2(w, o):
    # pkg/dem/Superquadrics.hpp:210-219
    _base(w, "SuperquadricsGeom", o)
    w.v2("curvatures1", o["curvatures1"])
    w.v2("curvatures2", o["curvatures2"])
    for k in ("curvatureAngle", "alpha", "K", "E", "curvatures_sum"):
        w.real(k, o[k])
    w.bool("isSphere", o["isSphere"])


def _norm_phys(w, o):
    _base(w, "IPhys", o)                 # pkg/common/NormShearPhys.hpp:10-12
    w.real("kn", o["kn"])
    w.v3("normalForce", o["normalForce"])


def _norm_shear_phys(w, o):
    _base(w, "NormPhys", o)              # pkg/common/NormShearPhys.hpp:22-25
    w.real("ks", o["ks"])
    w.v3("shearForce", o["shearForce"])


def _frict_phys(w, o):
    _base(w, "NormShearPhys", o)         # pkg/dem/FrictPhys.hpp:19-20
    w.real("tangensOfFrictionAngle", o["tangensOfFrictionAngle"])


def _sq_phys(w, o):
    # pkg/dem/Superquadrics.hpp:300-309
    _base(w, "FrictPhys", o)
    w.v3("normalViscous", o["normalViscous"])
    w.v3("shearViscous", o["shearViscous"])
    w.real("betan", o["betan"])
    w.real("betas", o["betas"])


def _sq_hm_phys(w, o):
    # pkg/dem/Superquadrics.hpp:313-324
    _base(w, "SuperquadricsPhys", o)
    for k in ("nuab", "Gab", "mu1", "mu2"):
        w.real(k, o[k])


def _interaction_container(w, o):
    # core/InteractionContainer.hpp:121
    _base(w, "Serializable", o)
    w.ptr_vector("interaction", "Interaction", o["interaction"])
    w.bool("serializeSorted", False)
    w.bool("dirty", o.get("dirty", False))


def _cell(w, o):
    # core/Cell.hpp:143-156
    _base(w, "Serializable", o)
    for k in ("trsf", "refHSize", "hSize", "prevHSize", "velGrad", "nextVelGrad", "prevVelGrad"):
        w.mat3(k, o[k])
    w.bool("homoDeform", o["homoDeform"])
    w.bool("velGradChanged", o["velGradChanged"])


_CLASSES = {
    "Serializable": _serializable, "Scene": _scene, "BodyContainer": _body_container,
    "NodeContainer": _node_container, "FEContainer": _fe_container, "EnergyTracker": _energy_tracker,
    "Body": _body, "State": _state, "Shape": _shape, "Superquadrics": _superquadrics, "Wall": _wall,
    "Bound": _bound, "Aabb": _aabb, "Material": _material, "SuperquadricsMat": _sq_mat,
    "SuperquadricsMat2": _sq_mat2, "Interaction": _interaction, "IGeom": _igeom, "IPhys": _iphys,
    "SuperquadricsGeom": _sq_geom, "SuperquadricsGeom2": _sq_geom2, "NormPhys": _norm_phys,
    "NormShearPhys": _norm_shear_phys, "FrictPhys": _frict_phys, "SuperquadricsPhys": _sq_phys,
    "SuperquadricsHertzMindlinPhys": _sq_hm_phys, "InteractionContainer": _interaction_container, "Cell": _cell,
}


def dumps(scene):
    """The archive text of a Scene object graph (SObj("Scene", ...))."""
    w = _Writer()
    w.sptr("scene", "Scene", scene)
    return w.text()


# ------------------------------------------------------------------------------------------
# Reader: generic decoding of the element tree (class names from class_id / class_name,
# shared objects from object_id / object_id_reference)
class Node:
    """A decoded element: the class name when the archive names it, its child values by tag
    (repeated tags, the ``item`` elements of containers, as a list)."""
    __slots__ = ("cls", "f")

    def __init__(self, cls):
        self.cls = cls
        self.f = {}

    def __getitem__(self, k):
        return self.f[k]

    def get(self, k, default=None):
        return self.f.get(k, default)


class _Null:
    pass


NULL = _Null()


def _decode(root):
    classes, objects = {}, {}
    stack = []
    result = None
    for ev, el in root:
        if ev == "start":
            a = el.attrib
            cls = None
            cid = a.get("class_id")
            if cid is not None:
                cid = int(cid)
                if cid == -1:
                    stack.append((el, NULL))
                    continue
                if "class_name" in a:
                    classes[cid] = a["class_name"]
                cls = classes.get(cid)
            elif "class_id_reference" in a:
                cls = classes.get(int(a["class_id_reference"]))
            ref = a.get("object_id_reference")
            if ref is not None:
                stack.append((el, ("ref", ref)))
                continue
            n = Node(cls)
            oid = a.get("object_id")
            if oid is not None:
                objects[oid] = n
            stack.append((el, n))
        else:
            el_, v = stack.pop()
            if v is NULL:
                val = None
            elif isinstance(v, tuple):
                val = objects[v[1]]
            elif not v.f and (len(el) == 0):
                # a leaf: primitive text, or an object without attributes (keeps its identity)
                val = v if (v.cls is not None or "object_id" in el.attrib) else (el.text or "")
            else:
                val = v
            el.clear()
            if stack:
                parent = stack[-1][1]
                if isinstance(parent, Node):
                    tag = el_.tag
                    if tag == "item":
                        parent.f.setdefault("item", []).append(val)
                    else:
                        parent.f[tag] = val
            else:
                result = val
    return result


def loads_tree(data):
    """Decode archive bytes into the tree of Nodes under the top-level ``scene`` element."""
    it = ET.iterparse(io.BytesIO(data), events=("start", "end"))
    # skip the boost_serialization wrapper element
    ev, top = next(it)
    if top.tag != "boost_serialization":
        raise ValueError("not a Boost.Serialization XML archive")

    def inner():
        depth = 0
        for ev, el in it:
            if ev == "start":
                depth += 1
            else:
                if depth == 0:
                    return
                depth -= 1
            yield ev, el
    return _decode(inner())


def _items(node):
    if node is None or isinstance(node, str):
        return []
    return node.get("item", [])


def _ptr(node):
    """The object a shared_ptr element points to (None for a null pointer)."""
    if node is None or isinstance(node, str):
        return None
    return node.get("px")


def _r(x):
    return _parse_real(x)


def _i(x):
    return int(x.strip())


def _vec(node, comps):
    return np.array([_r(node[c]) for c in comps])


def _v3(node):
    return _vec(node, ("x", "y", "z"))


def _v2(node):
    return _vec(node, ("x", "y"))


def _quat(node):
    return _vec(node, ("w", "x", "y", "z"))


def _mat3(node):
    return np.array([[_r(node["m%d%d" % (i, j)]) for j in range(3)] for i in range(3)])


def _chain(node, name):
    """Attributes of ``node`` and of its base-class elements, flattened, with the dynamic class
    name; ``name`` is the static class used when the archive does not name one."""
    out = {}
    cur = node
    while isinstance(cur, Node):
        base = None
        for k, v in cur.f.items():
            if k in _BASES and isinstance(v, Node) and not isinstance(v, str):
                base = v
            elif k not in out:
                out[k] = v
        cur = base
    return (node.cls or name), out


_BASES = ("Serializable", "Shape", "Bound", "Material", "SuperquadricsMat", "IGeom", "IPhys", "SuperquadricsGeom",
          "NormPhys", "NormShearPhys", "FrictPhys", "SuperquadricsPhys", "Engine", "GlobalEngine",
          "PartialEngine", "Collider", "Functor", "Dispatcher", "BoundFunctor", "IGeomFunctor", "IPhysFunctor",
          "LawFunctor", "PeriodicEngine")


# ------------------------------------------------------------------------------------------
# The scene in plain arrays
class ArchiveScene:
    """A scene read from or to be written to an archive, in plain arrays.

    bodies: ``kind`` (0 superquadric, 1 wall), ``shape5`` (rx, ry, rz, eps1, eps2),
    ``isSphere``, ``wall`` (axis, sense), ``mat`` (index into ``materials``), ``state`` in the
    engine's SQDEM_BODY_STRIDE layout (pos, ori w-x-y-z, vel, angVel, angMom, force, torque,
    bound min/max, bound refPos, sweepLength, lastUpdateIter, mass, inertia), ``hasBound``,
    ``blockedDOFs``, ``isDamped``, ``densityScaling``, ``refPos``, ``refOri``, ``groupMask``,
    ``flags``, ``clumpId``, ``chain``, ``iterBorn``, ``timeBorn``.
    interactions: ``intr`` in the engine's SQDEM_INTR_STRIDE layout (isReal = phys present,
    hasGeom = geom present), ``iterMadeReal``, ``iterBorn``, ``hm`` (SuperquadricsGeom2 /
    SuperquadricsHertzMindlinPhys), ``viscous`` (normalViscous, shearViscous), ``betas2``
    (betan, betas), ``hmPhys`` (nuab, Gab, mu1, mu2), ``points11`` (point11, point22).
    materials: list of dicts (``cls`` SuperquadricsMat or SuperquadricsMat2, id, label,
    density, Kn, Ks, frictionAngle, betan, betas, IsSplitable, strength[, G, nu]).
    cell: dict of Cell's attributes (3x3 arrays and two flags) or None when not periodic."""

    def __init__(self):
        self.dt = 1e-8
        self.iter = 0
        self.time = 0.0
        self.isPeriodic = False
        self.tags = []
        self.materials = []
        self.cell = None
        self.engines = []
        self.n = 0


def _material_obj(m, k):
    kw = dict(id=k, label=m.get("label", ""), density=float(m["density"]), Kn=float(m["Kn"]), Ks=float(m["Ks"]),
              frictionAngle=float(m["frictionAngle"]), betan=float(m["betan"]), betas=float(m["betas"]),
              IsSplitable=bool(m.get("IsSplitable", False)), strength=float(m.get("strength", 100.0)))
    if m.get("cls", "SuperquadricsMat") == "SuperquadricsMat2":
        return SObj("SuperquadricsMat2", G=float(m["G"]), nu=float(m["nu"]), **kw)
    return SObj("SuperquadricsMat", **kw)


def scene_graph(a):
    """The Scene object graph of an ArchiveScene, ready for dumps()."""
    mats = [_material_obj(m, k) for k, m in enumerate(a.materials)]
    bodies = []
    for i in range(a.n):
        st = a.state[i]
        look = dict(color=a.shapeColor[i], wire=bool(a.shapeWire[i]), highlight=bool(a.shapeHighlight[i]))
        if a.kind[i] == 1:
            shape = SObj("Wall", axis=int(a.wall[i, 0]), sense=int(a.wall[i, 1]), **look)
        else:
            rx, ry, rz, e1, e2 = (float(x) for x in a.shape5[i])
            shape = SObj("Superquadrics", rx=rx, ry=ry, rz=rz, eps1=e1, eps2=e2, isSphere=bool(a.isSphere[i]), **look)
        bound = None
        if a.hasBound[i]:
            bound = SObj("Aabb", lastUpdateIter=int(st[32]), refPos=st[28:31], sweepLength=float(st[31]),
                         color=a.boundColor[i])
        state = SObj("State", pos=st[0:3], ori=st[3:7], vel=st[7:10], mass=float(st[33]), angVel=st[10:13],
                     angMom=st[13:16], inertia=st[34:37], refPos=a.refPos[i], refOri=a.refOri[i],
                     blockedDOFs=int(a.blockedDOFs[i]), isDamped=bool(a.isDamped[i]),
                     densityScaling=float(a.densityScaling[i]))
        bodies.append(SObj("Body", id=i, groupMask=int(a.groupMask[i]), flags=int(a.flags[i]), material=mats[a.mat[i]],
                           state=state, shape=shape, bound=bound, intrs=[], clumpId=int(a.clumpId[i]),
                           chain=int(a.chain[i]), iterBorn=int(a.iterBorn[i]), timeBorn=float(a.timeBorn[i])))
    intrs = []
    for k in range(len(a.intr)):
        r = a.intr[k]
        i1, i2 = int(r[0]), int(r[1])
        geom = phys = None
        hm = bool(a.hm[k])
        if r[3]:
            g = dict(PenetrationDepth=float(r[4]), contactAngle=r[5:7], contactPoint=r[7:10], normal=r[10:13],
                     shearInc=r[13:16], point1=r[16:19], point2=r[19:22], isShearNew=bool(r[22]),
                     twist_axis=r[32:35], orthonormal_axis=r[35:38], relativeVn=r[38:41], relativeVs=r[41:44],
                     point11=a.points11[k, 0:3], point22=a.points11[k, 3:6])
            if hm:
                geom = SObj("SuperquadricsGeom2", curvatures1=r[47:49], curvatures2=r[49:51], curvatureAngle=float(r[51]),
                            alpha=float(r[52]), K=float(r[53]), E=float(r[54]), curvatures_sum=float(r[55]),
                            isSphere=bool(r[56]), **g)
            else:
                geom = SObj("SuperquadricsGeom", **g)
        if r[2]:
            p = dict(kn=float(r[23]), ks=float(r[24]), tangensOfFrictionAngle=float(r[25]), normalForce=r[26:29],
                     shearForce=r[29:32], normalViscous=a.viscous[k, 0:3], shearViscous=a.viscous[k, 3:6],
                     betan=float(a.betas2[k, 0]), betas=float(a.betas2[k, 1]))
            if hm:
                phys = SObj("SuperquadricsHertzMindlinPhys", nuab=float(a.hmPhys[k, 0]), Gab=float(a.hmPhys[k, 1]),
                            mu1=float(a.hmPhys[k, 2]), mu2=float(a.hmPhys[k, 3]), **p)
            else:
                phys = SObj("SuperquadricsPhys", **p)
        I = SObj("Interaction", id1=i1, id2=i2, iterMadeReal=int(a.iterMadeReal[k]), geom=geom, phys=phys,
                 cellDist=r[44:47].astype(np.int64), iterBorn=int(a.iterBorn_i[k]))
        intrs.append(I)
        bodies[i1].f["intrs"].append((i2, I))
        bodies[i2].f["intrs"].append((i1, I))
    for b in bodies:
        b.f["intrs"].sort(key=lambda kv: kv[0])
    if a.cell is not None:
        cell = SObj("Cell", **a.cell)
    else:
        I3 = np.eye(3)
        cell = SObj("Cell", trsf=I3, refHSize=I3, hSize=I3, prevHSize=I3, velGrad=np.zeros((3, 3)),
                    nextVelGrad=np.zeros((3, 3)), prevVelGrad=np.zeros((3, 3)), homoDeform=True, velGradChanged=False)
    return SObj("Scene", dt=a.dt, iter=a.iter, time=a.time, isPeriodic=a.isPeriodic, tags=list(a.tags),
                bodies=SObj("BodyContainer", body=bodies), interactions=SObj("InteractionContainer", interaction=intrs),
                materials=mats, cell=cell)


def save(path, a):
    """Write an ArchiveScene to ``path`` (.xml, .xml.bz2 or .xml.gz)."""
    if not is_xml_filename(path):
        raise ValueError("archive file names end in .xml, .xml.bz2 or .xml.gz (ObjectIO::isXmlFilename)")
    text = dumps(scene_graph(a))
    with _open(path, "wb") as f:
        f.write(text.encode("utf-8"))


def load(path):
    """Read an archive written by the reference's O.save or by save() into an ArchiveScene."""
    with _open(path, "rb") as f:
        data = f.read()
    return from_tree(loads_tree(data))


def from_tree(root):
    sc = _ptr(root)
    if sc is None:
        raise ValueError("the archive holds no scene")
    _, S = _chain(sc, "Scene")
    a = ArchiveScene()
    a.dt, a.iter, a.time = _r(S["dt"]), _i(S["iter"]), _r(S["time"])
    a.isPeriodic = _i(S["isPeriodic"]) != 0
    a.tags = [t for t in _items(S.get("tags"))]
    # materials: the shared ones, by their id (Material::id is the index in O.materials)
    mats = []
    mat_index = {}
    for k, mp in enumerate(_items(S.get("materials"))):
        m = _ptr(mp)
        cls, M = _chain(m, "Material")
        if cls not in ("SuperquadricsMat", "SuperquadricsMat2", "FrictMat"):
            raise ValueError(f"material class {cls} is not available on the superquadric path")
        d = {"cls": cls, "id": _i(M["id"]), "label": M.get("label") or "", "density": _r(M["density"])}
        if cls == "FrictMat":
            d.update(cls="SuperquadricsMat", Kn=_r(M["young"]), Ks=_r(M["young"]) * _r(M["poisson"]),
                     frictionAngle=_r(M["frictionAngle"]), betan=0.0, betas=0.0)
        else:
            for key in ("Kn", "Ks", "frictionAngle", "betan", "betas", "strength"):
                d[key] = _r(M[key])
            d["IsSplitable"] = _i(M["IsSplitable"]) != 0
            if cls == "SuperquadricsMat2":
                d["G"], d["nu"] = _r(M["G"]), _r(M["nu"])
        mats.append(d)
        mat_index[id(m)] = k
    bodies = [_ptr(x) for x in _items(_chain(_ptr(S["bodies"]), "BodyContainer")[1].get("body"))]
    if any(b is None for b in bodies):
        raise ValueError("the archive has erased bodies (null slots in O.bodies); renumber them before the GPU path")
    n = len(bodies)
    a.n = n
    a.kind = np.zeros(n, np.int32)
    a.shape5 = np.zeros((n, 5))
    a.isSphere = np.zeros(n, np.int32)
    a.wall = np.zeros((n, 2), np.int32)
    a.mat = np.zeros(n, np.int32)
    a.state = np.zeros((n, BODY_STRIDE))
    a.hasBound = np.zeros(n, bool)
    a.blockedDOFs = np.zeros(n, np.int64)
    a.isDamped = np.ones(n, bool)
    a.densityScaling = np.ones(n)
    a.refPos = np.zeros((n, 3))
    a.refOri = np.tile([1.0, 0, 0, 0], (n, 1))
    a.groupMask = np.ones(n, np.int64)
    a.flags = np.zeros(n, np.int64)
    a.clumpId = np.full(n, ID_NONE, np.int64)
    a.chain = np.full(n, -1, np.int64)
    a.iterBorn = np.full(n, -1, np.int64)
    a.timeBorn = np.full(n, -1.0)
    a.shapeColor = np.ones((n, 3))
    a.shapeWire = np.zeros(n, bool)
    a.shapeHighlight = np.zeros(n, bool)
    a.boundColor = np.ones((n, 3))
    intr_nodes = {}
    for i, b in enumerate(bodies):
        _, B = _chain(b, "Body")
        if _i(B["id"]) != i:
            raise ValueError(f"body {i} carries id {_i(B['id'])}")
        a.groupMask[i], a.flags[i] = _i(B["groupMask"]), _i(B["flags"])
        a.clumpId[i], a.chain[i] = _i(B["clumpId"]), _i(B["chain"])
        a.iterBorn[i], a.timeBorn[i] = _i(B["iterBorn"]), _r(B["timeBorn"])
        m = _ptr(B["material"])
        if m is None or id(m) not in mat_index:
            raise ValueError(f"body {i} has no shared material (O.materials)")
        a.mat[i] = mat_index[id(m)]
        cls, SH = _chain(_ptr(B["shape"]), "Shape")
        a.shapeColor[i] = _v3(SH["color"])
        a.shapeWire[i] = _i(SH["wire"]) != 0
        a.shapeHighlight[i] = _i(SH["highlight"]) != 0
        if cls == "Superquadrics":
            a.shape5[i] = (_r(SH["rx"]), _r(SH["ry"]), _r(SH["rz"]), _r(SH["eps1"]), _r(SH["eps2"]))
            rxyz, eps = _v3(SH["rxyz"]), _v2(SH["eps"])
            # Superquadrics::Initial takes rx..eps2 from rxyz and eps (Superquadrics.cpp:51-55)
            a.shape5[i] = (rxyz[0], rxyz[1], rxyz[2], eps[0], eps[1])
            a.isSphere[i] = _i(SH["isSphere"])
        elif cls == "Wall":
            a.kind[i] = 1
            a.wall[i] = (_i(SH["axis"]), _i(SH["sense"]))
        else:
            raise ValueError(f"shape class {cls} is not available on the superquadric path")
        _, ST = _chain(_ptr(B["state"]), "State")
        se3 = ST["se3"]
        st = a.state[i]
        st[0:3] = _v3(se3["position"])
        st[3:7] = _quat(se3["orientation"])
        st[7:10] = _v3(ST["vel"])
        st[10:13] = _v3(ST["angVel"])
        st[13:16] = _v3(ST["angMom"])
        st[22:28] = np.nan
        st[33] = _r(ST["mass"])
        st[34:37] = _v3(ST["inertia"])
        a.refPos[i] = _v3(ST["refPos"])
        a.refOri[i] = _quat(ST["refOri"])
        a.blockedDOFs[i] = _i(ST["blockedDOFs"])
        a.isDamped[i] = _i(ST["isDamped"]) != 0
        a.densityScaling[i] = _r(ST["densityScaling"])
        bd = _ptr(B["bound"])
        if bd is not None:
            _, BD = _chain(bd, "Bound")
            a.hasBound[i] = True
            a.boundColor[i] = _v3(BD["color"])
            st[28:31] = _v3(BD["refPos"])
            st[31] = _r(BD["sweepLength"])
            st[32] = _i(BD["lastUpdateIter"])
        else:
            st[28:31] = np.nan
        for kv in _items(B.get("intrs")):
            I = _ptr(kv["second"])
            if I is not None:
                intr_nodes[id(I)] = I
    # the saved interactions: the container's list (InteractionContainer::preSave)
    IC = _chain(_ptr(S["interactions"]), "InteractionContainer")[1]
    saved = [_ptr(x) for x in _items(IC.get("interaction"))]
    m = len(saved)
    a.intr = np.zeros((m, INTR_STRIDE))
    a.iterMadeReal = np.zeros(m, np.int64)
    a.iterBorn_i = np.zeros(m, np.int64)
    a.hm = np.zeros(m, bool)
    a.viscous = np.zeros((m, 6))
    a.betas2 = np.zeros((m, 2))
    a.hmPhys = np.zeros((m, 4))
    a.points11 = np.zeros((m, 6))
    for k, I in enumerate(saved):
        _, IN = _chain(I, "Interaction")
        r = a.intr[k]
        r[0], r[1] = _i(IN["id1"]), _i(IN["id2"])
        a.iterMadeReal[k], a.iterBorn_i[k] = _i(IN["iterMadeReal"]), _i(IN["iterBorn"])
        cd = IN["cellDist"]
        r[44:47] = (_i(cd["x"]), _i(cd["y"]), _i(cd["z"]))
        g = _ptr(IN["geom"])
        if g is not None:
            gcls, G = _chain(g, "IGeom")
            if gcls not in ("SuperquadricsGeom", "SuperquadricsGeom2"):
                raise ValueError(f"geometry class {gcls} is not available on the superquadric path")
            r[3] = 1
            r[4] = _r(G["PenetrationDepth"])
            r[5:7] = _v2(G["contactAngle"])
            r[7:10] = _v3(G["contactPoint"])
            r[10:13] = _v3(G["normal"])
            r[13:16] = _v3(G["shearInc"])
            r[16:19] = _v3(G["point1"])
            r[19:22] = _v3(G["point2"])
            r[22] = _i(G["isShearNew"])
            r[32:35] = _v3(G["twist_axis"])
            r[35:38] = _v3(G["orthonormal_axis"])
            r[38:41] = _v3(G["relativeVn"])
            r[41:44] = _v3(G["relativeVs"])
            a.points11[k] = np.r_[_v3(G["point11"]), _v3(G["point22"])]
            if gcls == "SuperquadricsGeom2":
                a.hm[k] = True
                r[47:49] = _v2(G["curvatures1"])
                r[49:51] = _v2(G["curvatures2"])
                r[51] = _r(G["curvatureAngle"])
                r[52], r[53], r[54], r[55] = _r(G["alpha"]), _r(G["K"]), _r(G["E"]), _r(G["curvatures_sum"])
                r[56] = _i(G["isSphere"])
        p = _ptr(IN["phys"])
        if p is not None:
            pcls, P = _chain(p, "IPhys")
            if pcls not in ("SuperquadricsPhys", "SuperquadricsHertzMindlinPhys", "FrictPhys"):
                raise ValueError(f"physics class {pcls} is not available on the superquadric path")
            r[2] = 1
            r[23], r[24], r[25] = _r(P["kn"]), _r(P["ks"]), _r(P["tangensOfFrictionAngle"])
            r[26:29] = _v3(P["normalForce"])
            r[29:32] = _v3(P["shearForce"])
            if pcls != "FrictPhys":
                a.viscous[k] = np.r_[_v3(P["normalViscous"]), _v3(P["shearViscous"])]
                a.betas2[k] = (_r(P["betan"]), _r(P["betas"]))
            if pcls == "SuperquadricsHertzMindlinPhys":
                a.hmPhys[k] = (_r(P["nuab"]), _r(P["Gab"]), _r(P["mu1"]), _r(P["mu2"]))
    a.materials = mats
    cp = _ptr(S.get("cell"))
    if a.isPeriodic and cp is not None:
        _, CL = _chain(cp, "Cell")
        a.cell = {k: _mat3(CL[k]) for k in ("trsf", "refHSize", "hSize", "prevHSize", "velGrad", "nextVelGrad",
                                              "prevVelGrad")}
        a.cell["homoDeform"] = _i(CL["homoDeform"]) != 0
        a.cell["velGradChanged"] = _i(CL["velGradChanged"]) != 0
    a.engines = [_engine_desc(_ptr(e)) for e in _items(S.get("engines"))]
    return a


def _engine_desc(e):
    """(class name, attributes) of an engine of an archive, the attribute values as text or
    nested descriptions; the scripting layer maps the engines it knows."""
    if e is None:
        return None
    cls, E = _chain(e, "Engine")

    def conv(v):
        if isinstance(v, Node):
            if "px" in v.f:
                return _engine_desc(v.f["px"])
            if "item" in v.f:
                return [conv(x) for x in v.f["item"]]
            if v.cls is None and not v.f:
                return None
            c, F = _chain(v, v.cls)
            return (c, {k: conv(x) for k, x in F.items() if k not in ("count", "item_version")})
        return v
    return (cls, {k: conv(v) for k, v in E.items()})


# ------------------------------------------------------------------------------------------
# Engines (sudodem_gb300.Engine) to and from archives
def _mat_dicts(materials, hm):
    m = materials
    out = []
    for k in range(len(m["Kn"])):
        d = {"cls": "SuperquadricsMat2" if ("G" in m or hm) else "SuperquadricsMat", "id": k, "label": "",
             "density": float(m["density"][k]), "Kn": float(m["Kn"][k]), "Ks": float(m["Ks"][k]),
             "frictionAngle": float(m["frictionAngle"][k]), "betan": float(m["betan"][k]),
             "betas": float(m["betas"][k]), "IsSplitable": False, "strength": 100.0}
        if d["cls"] == "SuperquadricsMat2":
            d["G"] = float(m["G"][k]) if "G" in m else 29e9
            d["nu"] = float(m["nu"][k]) if "nu" in m else 0.15
        out.append(d)
    return out


def from_engine(eng, spec, dt=None, time=None, tags=None, body_extra=None):
    """The ArchiveScene of an engine's current state.  ``spec`` is the SceneSpec the engine was
    loaded from (shapes and materials).  Written per interaction as the reference's functors
    would hold it: Ip2's betan/betas = max over the two materials and the Hertz-Mindlin
    coefficients nuab, Gab, mu1, mu2 (pkg/dem/Superquadrics.cpp:1111-1157, walls for id1 <= 5),
    normalViscous/shearViscous zero (the laws keep them in locals, Superquadrics.cpp:1229-1230),
    point11/point22 zero (drawing aids no functor sets).  iterMadeReal is not tracked by the
    GPU engine and is written as -1 (no superquadric functor reads it).  ``body_extra`` may give
    per-body ``refPos``, ``refOri``, ``groupMask``, ``blockedDOFs``, ``isDamped`` arrays."""
    st = eng.body_state()
    recs = eng.interactions(True)
    recs = recs[(recs[:, 2] != 0) | (recs[:, 3] != 0)]
    sc = eng.scalars()
    hm_model = eng.contact_model() == "hertz_mindlin"
    a = ArchiveScene()
    a.iter = int(sc[0])
    a.dt = float(spec.params["dt"] if dt is None else dt)
    a.time = a.iter * a.dt if time is None else float(time)
    a.isPeriodic = bool(spec.info.get("periodic"))
    a.tags = list(tags or [])
    a.materials = _mat_dicts(spec.materials, hm_model)
    n = len(spec.kind)
    a.n = n
    a.kind = np.asarray(spec.kind, np.int32).copy()
    a.shape5 = np.asarray(spec.shape5, np.float64).copy()
    a.isSphere = np.asarray(spec.isSphere, np.int32).copy()
    a.wall = np.asarray(spec.wall_axis_sense, np.int32).copy()
    a.mat = np.asarray(spec.mat, np.int32).copy()
    a.state = st.copy()
    a.hasBound = (a.kind == 0) | ~np.isnan(st[:, 28])
    ex = body_extra or {}
    wall = a.kind == 1
    a.blockedDOFs = np.asarray(ex.get("blockedDOFs", np.where(wall, DOF_ALL, 0)), np.int64)
    a.isDamped = np.asarray(ex.get("isDamped", np.ones(n, bool)), bool)
    a.densityScaling = np.ones(n)
    a.refPos = np.asarray(ex.get("refPos", np.where(wall[:, None], st[:, 0:3], 0.0)), np.float64)
    a.refOri = np.asarray(ex.get("refOri", np.tile([1.0, 0, 0, 0], (n, 1))), np.float64)
    a.groupMask = np.asarray(ex.get("groupMask", np.ones(n, np.int64)), np.int64)
    a.flags = np.where(wall, FLAG_BOUNDED, FLAG_BOUNDED | FLAG_ASPHERICAL).astype(np.int64)
    a.clumpId = np.full(n, ID_NONE, np.int64)
    a.chain = np.full(n, -1, np.int64)
    a.iterBorn = np.zeros(n, np.int64)
    a.timeBorn = np.zeros(n)
    a.shapeColor = np.asarray(ex.get("shapeColor", np.ones((n, 3))), np.float64)
    a.shapeWire = np.zeros(n, bool)
    a.shapeHighlight = np.zeros(n, bool)
    a.boundColor = np.ones((n, 3))
    m = len(recs)
    a.intr = recs.copy()
    a.iterMadeReal = np.full(m, -1, np.int64)
    a.iterBorn_i = np.full(m, a.iter, np.int64)
    a.hm = np.full(m, hm_model, bool)
    a.viscous = np.zeros((m, 6))
    a.points11 = np.zeros((m, 6))
    a.betas2 = np.zeros((m, 2))
    a.hmPhys = np.zeros((m, 4))
    mats = a.materials
    for k in range(m):
        i1, i2 = int(recs[k, 0]), int(recs[k, 1])
        m1, m2 = mats[a.mat[i1]], mats[a.mat[i2]]
        a.betas2[k] = (max(m1["betan"], m2["betan"]), max(m1["betas"], m2["betas"]))
        if hm_model and i1 > 5:
            a.hmPhys[k] = (0.5 * (m1["nu"] + m2["nu"]), 1.0 / ((1 - m1["nu"]) / m1["G"] + (1 - m2["nu"]) / m2["G"]),
                           1. / m1["G"] + 1. / m2["G"], m1["nu"] / m1["G"] + m2["nu"] / m2["G"])
    if a.isPeriodic:
        c = eng.cell()
        h = c[0:9].reshape(3, 3)
        vg = c[9:18].reshape(3, 3)
        a.cell = {"trsf": np.eye(3), "refHSize": h.copy(), "hSize": h.copy(), "prevHSize": h.copy(), "velGrad": vg.copy(),
                  "nextVelGrad": vg.copy(), "prevVelGrad": c[18:27].reshape(3, 3).copy(), "homoDeform": True,
                  "velGradChanged": False}
    return a


def spec_from_archive(a, params=None):
    """A SceneSpec of an ArchiveScene.  The archive carries dt but no engines: the other
    timestep parameters (gravity, damping, collider settings) come from ``params``."""
    from .assemblies import SceneSpec, default_params
    p = default_params()
    p.update(params or {})
    p["dt"] = a.dt
    ms = a.materials
    mats = {k: np.array([m[k] for m in ms], np.float64) for k in ("Kn", "Ks", "frictionAngle", "betan", "betas",
                                                                   "density")}
    hm = bool(np.any(a.hm))
    if hm or any(m["cls"] == "SuperquadricsMat2" for m in ms):
        mats["G"] = np.array([m.get("G", 29e9) for m in ms])
        mats["nu"] = np.array([m.get("nu", 0.15) for m in ms])
    info = {"contact_model": "hertz_mindlin" if hm else "linear"}
    if a.isPeriodic:
        if a.cell is None:
            raise ValueError("a periodic archive without a Cell")
        if not a.cell["homoDeform"]:
            raise NotImplementedError("Cell.homoDeform = False is not available on the GPU path")
        info.update(periodic=True, hSize=a.cell["hSize"].copy(),
                    velGrad=(a.cell["nextVelGrad"] if a.cell["velGradChanged"] else a.cell["velGrad"]).copy())
    st = a.state.copy()
    st[:, 16:28] = 0.0
    return SceneSpec(kind=a.kind.copy(), shape5=a.shape5.copy(), wall_axis_sense=a.wall.copy(), mat=a.mat.copy(),
                     isSphere=a.isSphere.copy(), state=st, materials=mats, params=p, info=info)


def to_engine(a, params=None, **engine_kw):
    """Build a GPU engine at the archive's state, with the reference's load semantics: bodies,
    bounds' sweep history (refPos, sweepLength, lastUpdateIter; min/max are not saved) and the
    saved interactions with their history are restored; the collider starts with a full sort
    at the next step, as InsertionSortCollider does after O.load (its sorted bounds are not
    part of the archive).  Returns (engine, spec)."""
    from ._native import Engine
    spec = spec_from_archive(a, params)
    eng = Engine(**engine_kw)
    eng.load(spec)
    st = a.state.copy()
    st[:, 22:28] = np.nan
    eng.put_body_state(st)
    if len(a.intr):
        eng.put_interactions(a.intr)
    s = eng.scalars()
    s[0] = a.iter
    s[8] = 0
    eng.put_scalars(s)
    if a.isPeriodic and a.cell is not None:
        c = eng.cell()
        c[18:27] = a.cell["prevVelGrad"].reshape(9)
        eng.put_cell(c)
    return eng, spec
