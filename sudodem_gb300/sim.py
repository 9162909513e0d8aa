"""SudoDEM3D-compatible scripting surface for the GPU engines.

A script written for SudoDEM3D's superellipsoid path runs unchanged::

    from sudodem_gb300.sim import *
    mat = SuperquadricsMat(Kn=1e5, Ks=5e4, frictionAngle=math.atan(0.5), density=2650)
    O.materials.append(mat)
    O.bodies.append(utils.wall(0, axis=2, sense=1, material=mat))
    b = NewSuperquadrics2(1e-3, 1e-3, 1e-3, 0.8, 1.2, mat, True, False)
    b.state.pos = (0, 0, 2e-3)
    O.bodies.append(b)
    O.engines = [ForceResetter(),
                 InsertionSortCollider([Bo1_Superquadrics_Aabb(), Bo1_Wall_Aabb()], verletDist=2e-4),
                 InteractionLoop([Ig2_Wall_Superquadrics_SuperquadricsGeom(),
                                  Ig2_Superquadrics_Superquadrics_SuperquadricsGeom()],
                                 [Ip2_SuperquadricsMat_SuperquadricsMat_SuperquadricsPhys()],
                                 [SuperquadricsLaw()]),
                 NewtonIntegrator(damping=0.3, gravity=(0, 0, -9.81), isSuperquadrics=1)]
    O.dt = 1e-6
    O.run(1000, True)

Classes, attribute names and defaults follow the reference:
  Omega / O            py/wrapper/sudodemWrapper.cpp:937-987
  Superquadrics        pkg/dem/Superquadrics.hpp:139-146
  SuperquadricsMat     pkg/dem/Superquadrics.hpp:247-264
  SuperquadricsMat2    pkg/dem/Superquadrics.hpp:266-277
  Wall                 pkg/common/Wall.hpp:11-13
  InsertionSortCollider pkg/common/InsertionSortCollider.hpp:212-222
  NewtonIntegrator     pkg/dem/NewtonIntegrator.hpp:70-89
  utils.wall           py/utils.py:311-327
  NewSuperquadrics*    py/_superquadrics_utils.cpp:251-380
The four engines run as one GPU timestep (libsqdem_gpu.so); PyRunner engines run on the
host between timesteps.  ``Ip2_FrictMat_FrictMat_FrictPhys`` and
``Law2_ScGeom_FrictPhys_CundallStrack`` are accepted as aliases of the superquadric
physics and law (FrictMat.young is read as the normal stiffness Kn and FrictMat.poisson as
Ks/Kn, the reading the ElastMat docstring gives, pkg/common/ElastMat.hpp:9).

The Hertz-Mindlin functor set -- Ig2_Wall_Superquadrics_SuperquadricsGeom2,
Ig2_Superquadrics_Superquadrics_SuperquadricsGeom2,
Ip2_SuperquadricsMat2_SuperquadricsMat2_HertzMindlinPhys and SuperquadricsLaw2 with
SuperquadricsMat2 materials -- selects the Nelder-Mead geometry and the Hertz-Mindlin law
(pkg/dem/Superquadrics_Ig2.cpp:2322-2700, pkg/dem/Superquadrics.cpp:1118-1557).  A plain
SuperquadricsMat under that set reads as SuperquadricsMat2 with the default G and nu.
"""
import math
import random as _random
import types

import numpy as np

from . import _native

__all__ = ["O", "Omega", "utils", "Body", "State", "Superquadrics", "Wall", "SuperquadricsMat", "FrictMat",
           "ForceResetter", "InsertionSortCollider", "Bo1_Superquadrics_Aabb", "Bo1_Wall_Aabb", "InteractionLoop",
           "Ig2_Superquadrics_Superquadrics_SuperquadricsGeom", "Ig2_Wall_Superquadrics_SuperquadricsGeom",
           "Ip2_SuperquadricsMat_SuperquadricsMat_SuperquadricsPhys", "SuperquadricsLaw",
           "Ip2_FrictMat_FrictMat_FrictPhys", "Law2_ScGeom_FrictPhys_CundallStrack", "NewtonIntegrator",
           "PyRunner", "CompressionEngine", "unbalancedForce", "getStress", "Cell", "NewSuperquadrics", "NewSuperquadrics2", "NewSuperquadrics_rot", "NewSuperquadrics_rot2",
           "Vector3", "Quaternion", "SuperquadricsMat2", "Ig2_Superquadrics_Superquadrics_SuperquadricsGeom2",
           "Ig2_Wall_Superquadrics_SuperquadricsGeom2", "Ip2_SuperquadricsMat2_SuperquadricsMat2_HertzMindlinPhys",
           "SuperquadricsLaw2"]


def Vector3(x=0.0, y=0.0, z=0.0):
    return np.array([x, y, z], dtype=np.float64)


def Quaternion(w=1.0, x=0.0, y=0.0, z=0.0):
    """Quaternion stored as (w, x, y, z)."""
    return np.array([w, x, y, z], dtype=np.float64)


class _Attr:
    """Keyword-attribute base mirroring SUDODEM_CLASS_BASE_DOC_ATTRS (lib/serialization/Serializable.hpp:205-227)."""
    _defaults = {}

    def __init__(self, **kw):
        for k, v in self._defaults.items():
            setattr(self, k, v() if callable(v) else v)
        for k, v in kw.items():
            if k not in self._defaults and k != "label":
                raise AttributeError(f"{type(self).__name__} has no attribute {k!r}")
            setattr(self, k, v)
        if not hasattr(self, "label"):
            self.label = ""

    def __repr__(self):
        return f"<{type(self).__name__}>"


# ----------------------------------------------------------------------------------------------
# Materials
class SuperquadricsMat(_Attr):
    _defaults = {"Kn": 1e8, "Ks": 1e5, "frictionAngle": 0.5, "betan": 0.0, "betas": 0.0, "density": 1000.0,
                 "IsSplitable": False, "strength": 100.0}


class SuperquadricsMat2(SuperquadricsMat):
    """SuperquadricsMat with the shear modulus G and Poisson's ratio nu of the Hertz-Mindlin model."""
    _defaults = dict(SuperquadricsMat._defaults, G=29e9, nu=0.15)


class FrictMat(_Attr):
    """FrictMat read through the alias mapping: young -> Kn, poisson -> Ks/Kn."""
    _defaults = {"young": 1e9, "poisson": 0.25, "frictionAngle": 0.5, "density": 1000.0}

    def as_superquadrics(self):
        return SuperquadricsMat(Kn=self.young, Ks=self.young * self.poisson, frictionAngle=self.frictionAngle,
                                density=self.density)


# ----------------------------------------------------------------------------------------------
# Shapes, state, bodies
class Superquadrics:
    """Superellipsoid (rx, ry, rz, eps1, eps2), Superquadrics.hpp:48-166."""

    def __init__(self, rx=1.0, ry=1.0, rz=1.0, eps1=1.0, eps2=1.0, isSphere=False):
        self.rx, self.ry, self.rz, self.eps1, self.eps2 = float(rx), float(ry), float(rz), float(eps1), float(eps2)
        self.isSphere = bool(isSphere)

    @property
    def rxyz(self):
        return Vector3(self.rx, self.ry, self.rz)

    @property
    def eps(self):
        return np.array([self.eps1, self.eps2])

    def _props(self):
        return _native.shape_props(self.rx, self.ry, self.rz, self.eps1, self.eps2)

    def getVolume(self):
        return float(self._props()[0])

    def getInertia(self):
        return self._props()[1:4].copy()

    def getr_max(self):
        return float(self._props()[4])


class Wall:
    """Axis-aligned plane (Wall.hpp:11-13): sense -1, 0 or +1."""

    def __init__(self, axis=0, sense=0):
        self.axis, self.sense = int(axis), int(sense)


class State:
    def __init__(self):
        self.pos = Vector3()
        self.ori = Quaternion()
        self.vel = Vector3()
        self.angVel = Vector3()
        self.angMom = Vector3()
        self.mass = 0.0
        self.inertia = Vector3()
        self.blockedDOFs = ""
        self.isDamped = True
        self.refPos = Vector3()

    def __setattr__(self, k, v):
        if k in ("pos", "vel", "angVel", "angMom", "inertia", "refPos", "ori"):
            v = np.array(v, dtype=np.float64)
        object.__setattr__(self, k, v)
        sc = getattr(self, "_scene", None)
        if sc is not None and k != "_scene":
            sc._hostDirty = True


_DOF = {"x": 1, "y": 2, "z": 4, "X": 8, "Y": 16, "Z": 32}


def _dof_mask(s):
    if isinstance(s, (int, np.integer)):
        return int(s)
    m = 0
    for ch in s:
        m |= _DOF[ch]
    return m


class Body:
    def __init__(self):
        self.id = -1
        self.shape = None
        self.state = State()
        self.mat = None
        self.material = None
        self.mask = 1
        self.aspherical = False
        self.bounded = True

    @property
    def dynamic(self):
        return _dof_mask(self.state.blockedDOFs) != 63

    def isStandalone(self):
        return True


# ----------------------------------------------------------------------------------------------
# Engines and functors (names and attributes of the reference)
class ForceResetter(_Attr):
    _defaults = {"dead": False}


class Bo1_Superquadrics_Aabb(_Attr):
    pass


class Bo1_Wall_Aabb(_Attr):
    pass


class InsertionSortCollider(_Attr):
    _defaults = {"verletDist": -0.5, "targetInterv": 50, "minSweepDistFactor": 0.1, "sortAxis": 0,
                 "doSort": False, "updatingDispFactor": -1.0, "sortThenCollide": False, "dead": False}

    def __init__(self, boundFunctors=None, **kw):
        super().__init__(**kw)
        self.boundFunctors = list(boundFunctors or [])


class Ig2_Superquadrics_Superquadrics_SuperquadricsGeom(_Attr):
    # GPU-only attribute: arithmetic form of the narrowphase ('fp64' or 'mixed')
    _defaults = {"precision": "fp64"}


class Ig2_Wall_Superquadrics_SuperquadricsGeom(_Attr):
    pass


class Ip2_SuperquadricsMat_SuperquadricsMat_SuperquadricsPhys(_Attr):
    pass


class SuperquadricsLaw(_Attr):
    pass


class Ip2_FrictMat_FrictMat_FrictPhys(Ip2_SuperquadricsMat_SuperquadricsMat_SuperquadricsPhys):
    """Alias with SuperquadricsPhys arithmetic (see the module docstring)."""


class Law2_ScGeom_FrictPhys_CundallStrack(SuperquadricsLaw):
    """Alias with SuperquadricsLaw arithmetic (see the module docstring)."""


class Ig2_Superquadrics_Superquadrics_SuperquadricsGeom2(_Attr):
    pass


class Ig2_Wall_Superquadrics_SuperquadricsGeom2(_Attr):
    pass


class Ip2_SuperquadricsMat2_SuperquadricsMat2_HertzMindlinPhys(_Attr):
    pass


class SuperquadricsLaw2(_Attr):
    pass


_LINEAR_SET = (Ig2_Superquadrics_Superquadrics_SuperquadricsGeom, Ig2_Wall_Superquadrics_SuperquadricsGeom,
               Ip2_SuperquadricsMat_SuperquadricsMat_SuperquadricsPhys, SuperquadricsLaw)
_HM_SET = (Ig2_Superquadrics_Superquadrics_SuperquadricsGeom2, Ig2_Wall_Superquadrics_SuperquadricsGeom2,
           Ip2_SuperquadricsMat2_SuperquadricsMat2_HertzMindlinPhys, SuperquadricsLaw2)


class InteractionLoop(_Attr):
    _defaults = {"dead": False}

    def __init__(self, geoms=None, physs=None, laws=None, **kw):
        super().__init__(**kw)
        self.geomDispatcher = list(geoms or [])
        self.physDispatcher = list(physs or [])
        self.lawDispatcher = list(laws or [])


class NewtonIntegrator(_Attr):
    _defaults = {"damping": 0.2, "gravity": (0.0, 0.0, 0.0), "isSuperquadrics": 0, "exactAsphericalRot": True,
                 "dead": False, "maxVelocitySq": float("nan"), "quiet_system_flag": False}


class CompressionEngine(_Attr):
    """Servo-controlled walls of a cubic specimen (pkg/dem/Compression.hpp:39-252): bodies 0-5 are
    the walls left, right, front, back, bottom, top.  Runs on the GPU between InteractionLoop and
    NewtonIntegrator.  Read-only results (UnbalancedForce, width, depth, height, strain,
    porosity) are refreshed after each run; recordData's file output is not written."""
    _defaults = {"cubic_specimen": True, "z_servo": True, "continueFlag": False, "shearMode": 1,
                 "wall_radius": 5.0, "wall_fix": True, "wall_radius0": 0.0, "gain_alpha": 0.5, "target_strain": 0.15,
                 "iterate_num_max": 100, "solve_num_max": 2000, "echo_interval": 1000, "ramp_interval": 10000,
                 "ramp_chunks": 400, "f_threshold": 0.01, "fmin_threshold": 0.01, "unbf_tol": 0.01,
                 "wall_max_vel": 1.0, "alpha": 0.5, "height0": 0.0, "width0": 0.0, "depth0": 0.0,
                 "height": 0.0, "width": 0.0, "depth": 0.0,
                 "left_wall_activated": True, "right_wall_activated": True, "front_wall_activated": True,
                 "back_wall_activated": True, "bottom_wall_activated": True, "top_wall_activated": True,
                 "hydroStrain": False, "hydroStrainRate": 0.0, "debug": False, "goalx": 0.0, "goaly": 0.0,
                 "goalz": 0.0, "savedata_interval": 12, "max_vel": 1.0, "externalWork": 0.0, "UnbalancedForce": 1.0,
                 "interStressControl": False, "file": "recordData", "dead": False,
                 "strain": (0.0, 0.0, 0.0), "porosity": 1.0}

    def _config(self):
        from .servo import servo_config
        if not self.cubic_specimen:
            raise NotImplementedError("CompressionEngine with a cylindrical wall is not available on the GPU path")
        kw = {k: float(getattr(self, k)) for k in (
            "z_servo", "continueFlag", "hydroStrain", "shearMode", "left_wall_activated", "right_wall_activated",
            "front_wall_activated", "back_wall_activated", "bottom_wall_activated", "top_wall_activated",
            "iterate_num_max", "solve_num_max", "echo_interval", "savedata_interval", "ramp_interval",
            "ramp_chunks", "goalx", "goaly", "goalz", "gain_alpha", "target_strain", "f_threshold",
            "fmin_threshold", "unbf_tol", "max_vel", "hydroStrainRate", "width0", "height0", "depth0")}
        return servo_config(enabled=1, **kw)

    def _absorb(self, st):
        from .servo import state_dict
        d = state_dict(st)
        a = self.__dict__
        a["UnbalancedForce"] = d["UnbalancedForce"]
        a["width"], a["depth"], a["height"] = d["width"], d["depth"], d["height"]
        a["width0"], a["depth0"], a["height0"] = d["width0"], d["depth0"], d["height0"]
        a["strain"] = (0.0, 0.0, d["strain2"])
        pv = d["particlesVolume"]
        a["porosity"] = 1.0 - pv / (d["width"] * d["depth"] * d["height"]) if pv > 0 and d["height"] else 1.0

    def getStress(self):
        """(mean stress, deviator stress) of the contact stress tensor in the box
        (Compression.cpp:764-841)."""
        eng = O._engine
        O.wait()
        st = eng.servo_state()
        from .servo import state_dict
        d = state_dict(st)
        vol = d["height"] * d["depth"] * d["width"]
        sig = -eng.get_stress(vol)
        mean = (sig[0, 0] + (sig[1, 1] + sig[2, 2])) / 3.0
        dev = sig - mean * np.eye(3)
        return (mean, float(np.sqrt(np.sum(dev * dev)) * np.sqrt(1.5)))


class PyRunner(_Attr):
    """Python command executed every iterPeriod steps (on the host, between timesteps)."""
    _defaults = {"command": "", "iterPeriod": 1, "initRun": False, "dead": False}

    def __init__(self, command="", iterPeriod=1, **kw):
        super().__init__(command=command, iterPeriod=iterPeriod, **kw)
        self.iterLast = 0


# ----------------------------------------------------------------------------------------------
# Containers
class BodyContainer:
    def __init__(self, scene):
        self._scene = scene
        self._b = []

    def append(self, b):
        if isinstance(b, (list, tuple)):
            return [self.append(x) for x in b]
        b.id = len(self._b)
        b.state._scene = self._scene
        self._b.append(b)
        self._scene._structDirty = True
        return b.id

    def __getitem__(self, i):
        self._scene._pull()
        return self._b[i]

    def __len__(self):
        return len(self._b)

    def __iter__(self):
        self._scene._pull()
        return iter(self._b)

    def clear(self):
        self._b = []
        self._scene._structDirty = True


class MaterialContainer(list):
    def append(self, m):
        super().append(m)
        return len(self) - 1

    def __getitem__(self, k):
        if isinstance(k, str):
            for m in self:
                if m.label == k:
                    return m
            raise KeyError(k)
        return super().__getitem__(k)


class _Geom:
    pass


class _Phys:
    pass


class Interaction:
    def __init__(self, rec):
        self.id1, self.id2 = int(rec[0]), int(rec[1])
        self._real = bool(rec[2])
        g = _Geom()
        g.penetrationDepth = g.PenetrationDepth = rec[4]
        g.contactAngle = rec[5:7].copy()
        g.contactPoint = rec[7:10].copy()
        g.normal = rec[10:13].copy()
        g.shearInc = rec[13:16].copy()
        g.point1, g.point2 = rec[16:19].copy(), rec[19:22].copy()
        g.isShearNew = bool(rec[22])
        p = _Phys()
        p.kn, p.ks, p.tangensOfFrictionAngle = rec[23], rec[24], rec[25]
        p.normalForce, p.shearForce = rec[26:29].copy(), rec[29:32].copy()
        # SuperquadricsGeom2 fields (zero under the linear model)
        g.curvatures1, g.curvatures2 = rec[47:49].copy(), rec[49:51].copy()
        g.curvatureAngle, g.alpha, g.K, g.E = rec[51], rec[52], rec[53], rec[54]
        g.curvatures_sum, g.isSphere = rec[55], bool(rec[56])
        self.geom = g if bool(rec[3]) else None
        self.phys = p if self._real else None

    def isReal(self):
        return self._real


class InteractionContainer:
    def __init__(self, scene):
        self._scene = scene

    def _recs(self):
        s = self._scene
        if s._engine is None:
            return np.zeros((0, _native.INTR_STRIDE))
        return s._engine.interactions(True)

    def __iter__(self):
        for r in self._recs():
            if r[2]:
                yield Interaction(r)

    def all(self):
        return [Interaction(r) for r in self._recs()]

    def __len__(self):
        return len(self._recs())

    def countReal(self):
        return int(np.sum(self._recs()[:, 2] != 0))

    def __getitem__(self, ids):
        a, b = ids
        for r in self._recs():
            if {int(r[0]), int(r[1])} == {a, b}:
                return Interaction(r)
        raise IndexError(f"no interaction {a}+{b}")


class ForceContainer:
    def __init__(self, scene):
        self._scene = scene

    def f(self, i):
        self._scene._pull()
        return self._scene._state[i, 16:19].copy()

    def t(self, i):
        self._scene._pull()
        return self._scene._state[i, 19:22].copy()


# ----------------------------------------------------------------------------------------------
class Cell:
    """Periodic cell (core/Cell.hpp): hSize columns are the base vectors; velGrad takes
    effect at the next integrator pass (Cell::setVelGrad); homoDeform is always on."""

    def __init__(self, scene):
        self._scene = scene
        self._hSize = np.eye(3)
        self._velGrad = np.zeros((3, 3))
        self._pending = None
        self.homoDeform = True

    def setBox(self, *size):
        if len(size) == 1:
            size = size[0]
        self.hSize = np.diag(np.array(size, dtype=np.float64))

    @property
    def hSize(self):
        e = self._scene._engine
        if e is not None and self._scene.periodic:
            return e.cell()[0:9].reshape(3, 3)
        return self._hSize.copy()

    @hSize.setter
    def hSize(self, m):
        self._hSize = np.array(m, dtype=np.float64).reshape(3, 3)
        self._scene._structDirty = True

    @property
    def size(self):
        h = self.hSize
        return np.linalg.norm(h, axis=0)

    @property
    def volume(self):
        return float(np.linalg.det(self.hSize))

    @property
    def velGrad(self):
        e = self._scene._engine
        if e is not None and self._scene.periodic:
            return e.cell()[9:18].reshape(3, 3)
        return self._velGrad.copy()

    @velGrad.setter
    def velGrad(self, m):
        m = np.array(m, dtype=np.float64).reshape(3, 3)
        self._velGrad = m
        e = self._scene._engine
        if e is not None and not self._scene._structDirty:
            e.set_velgrad(m)
        else:
            self._pending = m


class Omega:
    """The scene and its timestep loop (core/Omega.cpp, core/Scene.cpp:70-138)."""

    def __init__(self, device=0):
        self.device = device
        self.reset()

    def reset(self):
        self.bodies = BodyContainer(self)
        self.materials = MaterialContainer()
        self.interactions = InteractionContainer(self)
        self.forces = ForceContainer(self)
        self._engines = []
        self.dt = 1e-8
        self._engine = None
        self._structDirty = True
        self._hostDirty = False
        self._state = None
        self._pulled = True
        self._iter0 = 0
        self._timeBase = 0.0
        self._pendingArchive = None
        self.tags = {}
        self.periodic = False
        self.cell = Cell(self)

    # engines -------------------------------------------------------------------------------
    @property
    def engines(self):
        return self._engines

    @engines.setter
    def engines(self, e):
        self._engines = list(e)
        self._structDirty = True

    def _parse_engines(self):
        col = ilp = newton = servo = None
        runners = []
        for e in self._engines:
            if isinstance(e, ForceResetter):
                continue
            if isinstance(e, InsertionSortCollider):
                col = e
            elif isinstance(e, InteractionLoop):
                ilp = e
            elif isinstance(e, NewtonIntegrator):
                newton = e
            elif isinstance(e, CompressionEngine):
                if e.dead:
                    continue
                if ilp is None or newton is not None:
                    raise NotImplementedError("CompressionEngine runs on the GPU path only between InteractionLoop "
                                              "and NewtonIntegrator")
                servo = e
            elif isinstance(e, PyRunner):
                runners.append(e)
            else:
                raise NotImplementedError(f"engine {type(e).__name__} is not available on the GPU path")
        self._servo = servo
        if col is None or ilp is None or newton is None:
            raise RuntimeError("O.engines must contain InsertionSortCollider, InteractionLoop and NewtonIntegrator")
        functors = list(ilp.geomDispatcher) + list(ilp.physDispatcher) + list(ilp.lawDispatcher)
        for f in functors:
            if not isinstance(f, _LINEAR_SET + _HM_SET):
                raise NotImplementedError(f"functor {type(f).__name__} is not available on the GPU path")
        hm = [isinstance(f, _HM_SET) for f in functors]
        if any(hm) and not all(hm):
            raise NotImplementedError("the InteractionLoop mixes the linear (SuperquadricsGeom/Phys/Law) and the "
                                      "Hertz-Mindlin (SuperquadricsGeom2/HertzMindlinPhys/Law2) functor sets")
        self._contactModel = "hertz_mindlin" if functors and all(hm) else "linear"
        return col, ilp, newton, runners

    # state exchange --------------------------------------------------------------------------
    loadSkipped = ()

    def _material_table(self):
        mats, index = [], {}
        for b in self.bodies._b:
            m = b.mat if b.mat is not None else b.material
            if m is None:
                if not self.materials:
                    self.materials.append(SuperquadricsMat())
                m = self.materials[-1]
            if isinstance(m, int):
                m = self.materials[m]
            if isinstance(m, str):
                m = self.materials[m]
            if isinstance(m, FrictMat):
                key = id(m)
                if key not in index:
                    index[key] = len(mats)
                    mats.append(m.as_superquadrics())
                b._matIdx = index[key]
                continue
            if id(m) not in index:
                index[id(m)] = len(mats)
                mats.append(m)
            b._matIdx = index[id(m)]
        return mats

    def _body_arrays(self):
        n = len(self.bodies._b)
        kind = np.zeros(n, np.int32)
        shape5 = np.zeros((n, 5))
        was = np.zeros((n, 2), np.int32)
        mat = np.zeros(n, np.int32)
        sph = np.zeros(n, np.int32)
        st = np.zeros((n, _native.BODY_STRIDE))
        blocked = np.zeros(n, np.int32)
        for i, b in enumerate(self.bodies._b):
            s = b.state
            mat[i] = b._matIdx
            if isinstance(b.shape, Wall):
                kind[i] = 1
                was[i] = (b.shape.axis, b.shape.sense)
            elif isinstance(b.shape, Superquadrics):
                kind[i] = 0
                shape5[i] = (b.shape.rx, b.shape.ry, b.shape.rz, b.shape.eps1, b.shape.eps2)
                sph[i] = int(b.shape.isSphere)
            else:
                raise NotImplementedError(f"shape {type(b.shape).__name__} is not available on the GPU path")
            st[i, 0:3] = s.pos
            st[i, 3:7] = s.ori
            st[i, 7:10] = s.vel
            st[i, 10:13] = s.angVel
            st[i, 13:16] = s.angMom
            st[i, 28:31] = np.nan
            st[i, 33] = s.mass
            st[i, 34:37] = s.inertia
            blocked[i] = _dof_mask(s.blockedDOFs)
        return kind, shape5, was, mat, sph, st, blocked

    def _build(self):
        col, ilp, newton, runners = self._parse_engines()
        prec = "fp64"
        for g in ilp.geomDispatcher:
            if isinstance(g, Ig2_Superquadrics_Superquadrics_SuperquadricsGeom):
                prec = g.precision
        mats = self._material_table()
        kind, shape5, was, mat, sph, st, blocked = self._body_arrays()
        for i, b in enumerate(self.bodies._b):
            want = 63 if kind[i] == 1 else 0
            if blocked[i] != want:
                raise NotImplementedError("blockedDOFs other than the defaults (walls fixed, particles free) "
                                          "are not exposed through this surface yet")
        eng = _native.Engine(device=self.device, precision=prec)
        eng.set_materials([m.Kn for m in mats], [m.Ks for m in mats], [m.frictionAngle for m in mats],
                          [m.betan for m in mats], [m.betas for m in mats], [m.density for m in mats])
        d2 = SuperquadricsMat2._defaults
        eng.set_material_moduli([getattr(m, "G", d2["G"]) for m in mats], [getattr(m, "nu", d2["nu"]) for m in mats])
        eng.set_contact_model(self._contactModel)
        self._set_params(eng, col, newton)
        eng.set_bodies(kind, shape5, was, mat, sph, st)
        if self.periodic:
            vg = self.cell._pending if self.cell._pending is not None else self.cell._velGrad
            eng.set_periodic(self.cell._hSize, vg if np.any(vg != 0) else None)
            self.cell._pending = None
        if self._servo is not None:
            eng.set_servo(self._servo._config())
            self._servoKey = tuple(self._servo._config())
        if self._pendingArchive is not None:
            self._apply_archive(eng, self._pendingArchive)
            self._pendingArchive = None
        self._engine = eng
        self._parts = (col, ilp, newton, runners)
        self._structDirty = False
        self._hostDirty = False
        self._pulled = False

    def _set_params(self, eng, col, newton):
        eng.set_params(dt=self.dt, gravity=tuple(float(x) for x in newton.gravity), damping=newton.damping,
                       verletDist=col.verletDist, targetInterv=col.targetInterv,
                       minSweepDistFactor=col.minSweepDistFactor, sortAxis=col.sortAxis,
                       isSuperquadrics=newton.isSuperquadrics if newton.isSuperquadrics else 1,
                       exactAsphericalRot=int(newton.exactAsphericalRot))
        self._paramsKey = self._params_key(col, newton)

    def _params_key(self, col, newton):
        return (self.dt, tuple(newton.gravity), newton.damping, col.verletDist, col.targetInterv,
                col.minSweepDistFactor, col.sortAxis, newton.exactAsphericalRot)

    def _push(self):
        """Upload host-side modifications of body states."""
        st = self._engine.body_state()
        for i, b in enumerate(self.bodies._b):
            s = b.state
            st[i, 0:3] = s.pos
            st[i, 3:7] = s.ori
            st[i, 7:10] = s.vel
            st[i, 10:13] = s.angVel
            st[i, 13:16] = s.angMom
        self._engine.put_body_state(st)
        self._hostDirty = False

    def _pull(self):
        """Copy the GPU state into the Python body objects (after a run)."""
        if self._engine is None or self._pulled:
            return
        st = self._engine.body_state()
        self._state = st
        for i, b in enumerate(self.bodies._b):
            s = b.state
            d = s.__dict__
            d["pos"], d["ori"], d["vel"] = st[i, 0:3].copy(), st[i, 3:7].copy(), st[i, 7:10].copy()
            d["angVel"], d["angMom"] = st[i, 10:13].copy(), st[i, 13:16].copy()
        self._pulled = True

    # running ---------------------------------------------------------------------------------
    @property
    def iter(self):
        if self._engine is None:
            return self._iter0
        return int(self._engine.scalars()[0])

    @property
    def time(self):
        return self._timeBase + (self.iter - self._iter0) * self.dt

    def _prepare(self):
        if self._structDirty or self._engine is None:
            self._build()
        elif self._hostDirty:
            self._pull()
            self._push()
        col, ilp, newton, runners = self._parts
        if self._params_key(col, newton) != self._paramsKey:
            self._set_params(self._engine, col, newton)
        eng = self._engine
        st = eng.servo_state()
        if self._servo is not None:
            key = tuple(self._servo._config())
            if key != self._servoKey:   # attributes changed: new configuration, same engine state
                eng.set_servo(np.array(key))
                eng.put_servo(st)
                self._servoKey = key
        if st[34] >= 0:        # O.run(n) sets Scene::stopAtIter = iter + n (sudodemWrapper.cpp:739)
            st = st.copy()
            st[34] = -1
            eng.put_servo(st)
        if newton.quiet_system_flag:
            eng.set_quiet(True)
            newton.quiet_system_flag = False

    def step(self):
        self.run(1, True)

    def run(self, nSteps=1, wait=True):
        """Advance nSteps timesteps (PyRunner commands run between steps on the host)."""
        self._prepare()
        col, ilp, newton, runners = self._parts
        runners = [r for r in runners if not r.dead]
        done = 0
        while done < nSteps:
            it = self.iter
            chunk = nSteps - done
            for r in runners:
                nxt = r.iterPeriod - (it % r.iterPeriod) if r.iterPeriod > 0 else chunk
                chunk = min(chunk, max(1, nxt))
            self._engine.step(chunk)
            done += chunk
            self._pulled = False
            if runners:
                self._engine.sync()
                it = self.iter
                for r in runners:
                    if r.iterPeriod > 0 and it % r.iterPeriod == 0:
                        import __main__
                        exec(r.command, __main__.__dict__)
                        r.iterLast = it
                if self._structDirty or self._hostDirty:
                    self._prepare()
        if wait:
            self.report = self._engine.sync()
            self._after()

    def _after(self):
        if self._servo is not None:
            self._servo._absorb(self._engine.servo_state())

    def wait(self):
        if self._engine is not None:
            self.report = self._engine.sync()
            self._after()

    # saving and loading ------------------------------------------------------------------------
    def save(self, fileName):
        """Save the scene (O.save, core/Omega.cpp:230-279).

        A name ending in .xml, .xml.bz2 or .xml.gz (ObjectIO::isXmlFilename) writes the
        reference's Boost XML archive (sudodem_gb300.archive): bodies, materials, interactions
        with their history, cell, dt, iter, time and tags, which SudoDEM3D's O.load reads.  The
        engine list is written empty there: set O.engines after loading, in either program.
        Any other name writes this library's own format: the Python objects (bodies, materials,
        engines, cell) and the GPU state (sqdem_snapshot: contact history, collider and engine
        state), from which load() continues bit for bit."""
        from . import archive
        if archive.is_xml_filename(fileName):
            return self._save_archive(fileName)
        import pickle
        if self._engine is None or self._structDirty or self._hostDirty:
            self._prepare()
        self.wait()
        self._pull()
        blob = self._engine.snapshot()
        bodies = self.bodies._b
        scenes = [b.state.__dict__.pop("_scene", None) for b in bodies]
        try:
            payload = {"version": 1, "blob": blob, "bodies": bodies, "materials": list(self.materials),
                       "engines": self._engines, "dt": self.dt, "periodic": self.periodic, "tags": self.tags,
                       "cell": (self.cell._hSize, self.cell._velGrad), "device": self.device}
            with open(fileName, "wb") as f:
                pickle.dump(payload, f)
        finally:
            for bd, sc in zip(bodies, scenes):
                if sc is not None:
                    bd.state.__dict__["_scene"] = sc

    def load(self, fileName):
        """Load a scene written by save() (the run continues bit for bit from where it was saved)
        or a SudoDEM3D XML archive (.xml, .xml.bz2, .xml.gz; see save()).  From an archive, the
        engines the GPU path knows are mapped (ForceResetter, InsertionSortCollider,
        InteractionLoop with the superquadric functors, NewtonIntegrator, CompressionEngine,
        PyRunner); O.loadSkipped lists the others.  The collider starts with a full sort, as
        after the reference's O.load."""
        from . import archive
        if archive.is_xml_filename(fileName):
            return self._load_archive(fileName)
        import pickle
        with open(fileName, "rb") as f:
            d = pickle.load(f)
        if not isinstance(d, dict) or d.get("version") != 1:
            raise ValueError("not a scene saved by this library")
        self.reset()
        self.device = d["device"]
        for m in d["materials"]:
            self.materials.append(m)
        for bd in d["bodies"]:
            self.bodies.append(bd)
        self._engines = list(d["engines"])
        self.dt = d["dt"]
        self.periodic = d["periodic"]
        self.tags = d["tags"]
        self.cell._hSize, self.cell._velGrad = d["cell"]
        col, ilp, newton, runners = self._parse_engines()
        prec = "fp64"
        for g in ilp.geomDispatcher:
            if isinstance(g, Ig2_Superquadrics_Superquadrics_SuperquadricsGeom):
                prec = g.precision
        self._material_table()
        eng = _native.Engine(device=self.device, precision=prec)
        eng.restore(d["blob"])
        self._engine = eng
        self._parts = (col, ilp, newton, runners)
        self._paramsKey = self._params_key(col, newton)
        if self._servo is not None:
            self._servoKey = tuple(self._servo._config())
        self._structDirty = False
        self._hostDirty = False
        self._pulled = False


    # SudoDEM3D XML archives ---------------------------------------------------------------
    def _spec(self):
        """The SceneSpec of the current Python scene (shapes, materials, parameters)."""
        from .assemblies import SceneSpec, default_params
        mats = self._material_table()
        kind, shape5, was, mat, sph, st, blocked = self._body_arrays()
        m = {k: np.array([float(getattr(x, k)) for x in mats]) for k in ("Kn", "Ks", "frictionAngle", "betan",
                                                                            "betas", "density")}
        if any(isinstance(x, SuperquadricsMat2) for x in mats):
            d2 = SuperquadricsMat2._defaults
            m["G"] = np.array([float(getattr(x, "G", d2["G"])) for x in mats])
            m["nu"] = np.array([float(getattr(x, "nu", d2["nu"])) for x in mats])
        p = default_params()
        p["dt"] = self.dt
        info = {"contact_model": getattr(self, "_contactModel", "linear")}
        if self.periodic:
            info.update(periodic=True, hSize=self.cell._hSize.copy(), velGrad=self.cell._velGrad.copy())
        return SceneSpec(kind=kind, shape5=shape5, wall_axis_sense=was, mat=mat, isSphere=sph, state=st,
                         materials=m, params=p, info=info), mats

    def _save_archive(self, fileName):
        from . import archive
        if self._engine is None or self._structDirty or self._hostDirty:
            self._prepare()
        self.wait()
        self._pull()
        spec, mats = self._spec()
        bodies = self.bodies._b
        extra = {"refPos": np.array([np.asarray(b.state.refPos, dtype=np.float64) for b in bodies]).reshape(-1, 3),
                 "groupMask": np.array([int(b.mask) for b in bodies]),
                 "blockedDOFs": np.array([_dof_mask(b.state.blockedDOFs) for b in bodies]),
                 "isDamped": np.array([bool(b.state.isDamped) for b in bodies])}
        tags = [f"{k}={v}" for k, v in self.tags.items()]
        a = archive.from_engine(self._engine, spec, dt=self.dt, time=self.time, tags=tags, body_extra=extra)
        for k, x in enumerate(mats):
            a.materials[k]["label"] = str(getattr(x, "label", "") or "")
            a.materials[k]["IsSplitable"] = bool(getattr(x, "IsSplitable", False))
            a.materials[k]["strength"] = float(getattr(x, "strength", 100.0))
        archive.save(fileName, a)

    def _load_archive(self, fileName):
        from . import archive
        a = archive.load(fileName)
        device = self.device
        self.reset()
        self.device = device
        for k, m in enumerate(a.materials):
            cls = SuperquadricsMat2 if m["cls"] == "SuperquadricsMat2" else SuperquadricsMat
            kw = {x: m[x] for x in ("Kn", "Ks", "frictionAngle", "betan", "betas", "density")}
            if cls is SuperquadricsMat2:
                kw.update(G=m["G"], nu=m["nu"])
            mat = cls(IsSplitable=m.get("IsSplitable", False), strength=m.get("strength", 100.0), **kw)
            mat.label = m.get("label", "")
            self.materials.append(mat)
        for i in range(a.n):
            b = Body()
            if a.kind[i] == 1:
                b.shape = Wall(axis=int(a.wall[i, 0]), sense=int(a.wall[i, 1]))
            else:
                b.shape = Superquadrics(*a.shape5[i], isSphere=bool(a.isSphere[i]))
            b.mat = b.material = self.materials[int(a.mat[i])]
            b.mask = int(a.groupMask[i])
            b.aspherical = bool(a.flags[i] & archive.FLAG_ASPHERICAL)
            st = a.state[i]
            s = b.state
            s.pos, s.ori, s.vel = st[0:3].copy(), st[3:7].copy(), st[7:10].copy()
            s.angVel, s.angMom = st[10:13].copy(), st[13:16].copy()
            s.mass, s.inertia = float(st[33]), st[34:37].copy()
            s.refPos = a.refPos[i].copy()
            s.blockedDOFs = int(a.blockedDOFs[i])
            s.isDamped = bool(a.isDamped[i])
            self.bodies.append(b)
        self.dt = a.dt
        self._iter0 = a.iter
        self._timeBase = a.time
        self.tags = dict(t.split("=", 1) if "=" in t else (t, "") for t in a.tags)
        self.periodic = a.isPeriodic
        if a.isPeriodic and a.cell is not None:
            self.cell._hSize = a.cell["hSize"].copy()
            self.cell._velGrad = (a.cell["nextVelGrad"] if a.cell["velGradChanged"] else a.cell["velGrad"]).copy()
        self._engines, self.loadSkipped = _engines_from_archive(a.engines)
        self._pendingArchive = a
        self._structDirty = True

    def _apply_archive(self, eng, a):
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


def _num(v, default=0.0):
    try:
        return float(v)
    except (TypeError, ValueError):
        return default


def _vec3(v):
    if isinstance(v, tuple) and len(v) == 2 and isinstance(v[1], dict):
        return tuple(_num(v[1].get(c)) for c in ("x", "y", "z"))
    return None


def _functors(disp):
    """The functor class names of a dispatcher description (class, attributes)."""
    if not (isinstance(disp, tuple) and len(disp) == 2):
        return []
    out = []
    for f in disp[1].get("functors") or []:
        if isinstance(f, tuple) and f[0] in globals():
            out.append(globals()[f[0]]())
    return out


def _engines_from_archive(descs):
    """Map the engines of a SudoDEM3D archive onto this module's engine classes."""
    engines, skipped = [], []
    for d in descs:
        if d is None:
            continue
        cls, at = d
        dead = _num(at.get("dead"), 0) != 0
        if cls == "ForceResetter":
            engines.append(ForceResetter(dead=dead))
        elif cls == "InsertionSortCollider":
            e = InsertionSortCollider(_functors(at.get("boundDispatcher")))
            for k in ("verletDist", "minSweepDistFactor", "updatingDispFactor"):
                if k in at:
                    setattr(e, k, _num(at[k]))
            for k in ("targetInterv", "sortAxis"):
                if k in at:
                    setattr(e, k, int(_num(at[k])))
            engines.append(e)
        elif cls == "InteractionLoop":
            engines.append(InteractionLoop(_functors(at.get("geomDispatcher")), _functors(at.get("physDispatcher")),
                                           _functors(at.get("lawDispatcher"))))
        elif cls == "NewtonIntegrator":
            e = NewtonIntegrator()
            if "damping" in at:
                e.damping = _num(at["damping"])
            g = _vec3(at.get("gravity"))
            if g is not None:
                e.gravity = g
            if "isSuperquadrics" in at:
                e.isSuperquadrics = int(_num(at["isSuperquadrics"]))
            if "exactAsphericalRot" in at:
                e.exactAsphericalRot = _num(at["exactAsphericalRot"]) != 0
            engines.append(e)
        elif cls == "PyRunner":
            engines.append(PyRunner(command=at.get("command") or "", iterPeriod=int(_num(at.get("iterPeriod"), 1)),
                                    dead=dead))
        elif cls == "CompressionEngine":
            e = CompressionEngine()
            for k, v in CompressionEngine._defaults.items():
                if k in at and isinstance(v, (bool, int, float)) and not isinstance(at[k], tuple):
                    setattr(e, k, type(v)(_num(at[k])) if not isinstance(v, bool) else _num(at[k]) != 0)
            engines.append(e)
        else:
            skipped.append(cls)
    return engines, skipped


O = Omega()


# ----------------------------------------------------------------------------------------------
# Body factories
def _common_body(b, mat):
    b.mat = mat
    b.material = mat
    return b


def _mat_obj(mat):
    if isinstance(mat, int):
        return O.materials[mat]
    if isinstance(mat, str):
        return O.materials[mat]
    if mat is None:
        if not O.materials:
            O.materials.append(SuperquadricsMat())
        return O.materials[-1]
    return mat


def _density(m):
    return m.density


def NewSuperquadrics_rot2(x, y, z, ep1, ep2, mat, q0, q1, q2, q3, isSphere=False):
    """Superquadric body with a given orientation quaternion (py/_superquadrics_utils.cpp:354-380)."""
    m = _mat_obj(mat)
    b = _common_body(Body(), m)
    b.shape = Superquadrics(x, y, z, ep1, ep2, isSphere)
    props = b.shape._props()
    b.state.mass = _density(m) * props[0]
    b.state.inertia = props[1:4] * _density(m)
    b.aspherical = True
    q = np.array([q0, q1, q2, q3], dtype=np.float64)
    w, xx, yy, zz = q
    n = math.sqrt((xx * xx + yy * yy) + (zz * zz + w * w))
    b.state.ori = q / n
    return b


def NewSuperquadrics_rot(x, y, z, ep1, ep2, mat, q0, q1, q2, q3):
    return NewSuperquadrics_rot2(x, y, z, ep1, ep2, mat, q0, q1, q2, q3, False)


def NewSuperquadrics2(x, y, z, ep1, ep2, mat, rotate=False, isSphere=False):
    """Superquadric body (py/_superquadrics_utils.cpp:289-325).  With rotate=True the
    orientation is normalize(Identity + q(heading, attitude, bank)) for three uniform random
    Euler angles, as the reference does; Python's seeded ``random`` replaces C rand()."""
    if rotate:
        h, a, bk = (_random.random() * 2.0 * math.pi for _ in range(3))
        c1, s1 = math.cos(h / 2), math.sin(h / 2)
        c2, s2 = math.cos(a / 2), math.sin(a / 2)
        c3, s3 = math.cos(bk / 2), math.sin(bk / 2)
        c1c2, s1s2 = c1 * c2, s1 * s2
        w = c1c2 * c3 - s1s2 * s3
        qx = c1c2 * s3 + s1s2 * c3
        qy = s1 * c2 * c3 + c1 * s2 * s3
        qz = c1 * s2 * c3 - s1 * c2 * s3
        return NewSuperquadrics_rot2(x, y, z, ep1, ep2, mat, 1.0 + w, qx, qy, qz, isSphere)
    return NewSuperquadrics_rot2(x, y, z, ep1, ep2, mat, 1.0, 0.0, 0.0, 0.0, isSphere)


def NewSuperquadrics(x, y, z, ep1, ep2, mat, rotate=False):
    return NewSuperquadrics2(x, y, z, ep1, ep2, mat, rotate, False)


def _wall(position, axis, sense=0, color=None, material=-1, mask=1):
    """Fixed axis-aligned wall body (py/utils.py:311-327)."""
    b = Body()
    b.shape = Wall(axis=axis, sense=sense)
    if isinstance(position, (int, float)):
        p = Vector3()
        p[axis] = position
    else:
        p = np.array(position, dtype=np.float64)
    if isinstance(material, int) and material < 0:
        if not O.materials:
            O.materials.append(SuperquadricsMat())
        m = O.materials[material]
    else:
        m = _mat_obj(material)
    _common_body(b, m)
    b.state.pos = p
    b.state.refPos = p
    b.state.blockedDOFs = "xyzXYZ"
    b.aspherical = False
    b.mask = mask
    return b


def _avgNumInteractions(cutoff=0.0, skipFree=False, considerClumps=False):
    """Average number of real touching interactions per particle (cf. py/utils.py:498)."""
    recs = O.interactions._recs()
    parts = [b.id for b in O.bodies._b if isinstance(b.shape, Superquadrics)]
    touch = recs[(recs[:, 2] != 0) & (recs[:, 4] > 0)]
    cnt = {i: 0 for i in parts}
    for r in touch:
        for k in (int(r[0]), int(r[1])):
            if k in cnt:
                cnt[k] += 1
    vals = list(cnt.values())
    if skipFree:
        vals = [v for v in vals if v > 0]
    return 2.0 * len(touch) / max(len(parts), 1) if not skipFree else (sum(vals) / max(len(vals), 1))


def _unbalancedForce(useMaxForce=False):
    """Shop::unbalancedForce (py/_utils.cpp:428,570; pkg/dem/Shop_01.cpp:148-188)."""
    O.wait()
    return O._engine.unbalanced_force(bool(useMaxForce))


def _getStress(volume=0):
    """Shop::getStress (py/_utils.cpp:592; pkg/dem/Shop_02.cpp:350-376), 3x3."""
    O.wait()
    return O._engine.get_stress(float(volume))


utils = types.SimpleNamespace(wall=_wall, avgNumInteractions=_avgNumInteractions, unbalancedForce=_unbalancedForce,
                              getStress=_getStress)
unbalancedForce = _unbalancedForce
getStress = _getStress
