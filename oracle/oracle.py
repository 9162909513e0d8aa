"""ctypes wrapper of the CPU oracle (oracle/sqdem_oracle.cpp).

Test infrastructure only: imported by tests/, __graft_entry__.smoke() and bench.py's CPU
baseline.  Parity of the oracle against the reference is unpinned (the reference cannot be
built here and ships no golden data for this path); see the header of sqdem_oracle.cpp.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libsqdem_oracle.so")
BODY_STRIDE = 37
INTR_STRIDE = 57

_lib = None


def build(force=False):
    src = os.path.join(HERE, "sqdem_oracle.cpp")
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-B" if force else "-s", "-C", HERE], check=True)
    return LIB


def lib():
    global _lib
    if _lib is not None:
        return _lib
    build()
    L = C.CDLL(LIB)
    d, i, l, v = C.c_double, C.c_int, C.c_long, C.c_void_p
    dp = C.POINTER(d)
    sig = {
        "sqo_create": (v, []), "sqo_destroy": (None, [v]), "sqo_set_threads": (None, [v, i]),
        "sqo_add_material": (i, [v, d, d, d, d, d, d]),
        "sqo_add_wall": (i, [v, dp, i, i, i]),
        "sqo_add_sq": (i, [v, d, d, d, d, d, i, dp, i, dp]),
        "sqo_set_params": (None, [v, d, dp, d, d, i, d, i]),
        "sqo_step": (None, [v, i]), "sqo_collide": (i, [v]), "sqo_last_step_collided": (i, [v]),
        "sqo_iter": (l, [v]), "sqo_num_bodies": (i, [v]), "sqo_num_interactions": (l, [v]),
        "sqo_stats": (None, [v, C.POINTER(l)]), "sqo_max_velocity_sq": (d, [v]),
        "sqo_get_bodies": (None, [v, dp]), "sqo_set_bodies": (None, [v, dp]),
        "sqo_get_interactions": (None, [v, dp]), "sqo_set_interactions": (None, [v, l, dp]),
        "sqo_get_margins": (None, [v, dp]),
        "sqo_disfunction": (None, [dp, dp, dp, dp, dp, dp, d, d, dp, dp]),
        "sqo_lmder2": (None, [dp, dp, dp, dp, dp, dp, dp, dp]),
        "sqo_set_periodic_fix": (None, [v, i]),
        "sqo_set_math_noise": (None, [C.c_ulonglong, d]),
        "sqo_get_scalars": (None, [v, dp]), "sqo_set_scalars": (None, [v, dp]),
        "sqo_rebuild_sorted_bounds": (None, [v]),
        "sqo_pair_geom": (i, [v, i, i, i, dp, dp]),
        "sqo_eval_hist": (None, [v, C.POINTER(l)]),
        "sqo_set_servo": (None, [v, dp]), "sqo_get_servo": (None, [v, dp]), "sqo_put_servo": (None, [v, dp]),
        "sqo_set_quiet": (None, [v, C.c_int]), "sqo_unbalanced_force": (d, [v, C.c_int]),
        "sqo_get_stress": (None, [v, d, dp]),
        "sqo_set_periodic": (None, [v, dp, dp]), "sqo_set_velgrad": (None, [v, dp]),
        "sqo_get_cell": (None, [v, dp]), "sqo_set_cell": (None, [v, dp]),
        "sqo_shape_props": (None, [d, d, d, d, d, dp]),
        "sqo_surface": (None, [d, d, d, d, d, d, d, dp]),
        "sqo_normal": (None, [d, d, d, d, d, d, d, dp]),
        "sqo_normal2phi": (None, [d, d, d, d, d, dp, dp]),
        "sqo_set_contact_model": (None, [v, i]), "sqo_set_moduli": (None, [v, i, d, d]),
        "sqo_stats_nan_forces": (None, [v, C.POINTER(l)]),
        "sqo_pair_geom2": (i, [v, i, i, i, dp, dp]),
        "sqo_curvatures": (None, [d, d, d, d, d, d, d, dp]),
        "sqo_hertz_mindlin": (None, [dp, dp, d, dp]),
        "sqo_set_frozen": (None, [v, i]), "sqo_signature": (C.c_ulonglong, [v]), "sqo_reset_phys": (None, [v]),
        "sqo_set_material": (None, [v, i, d, d, d]), "sqo_set_eps": (None, [v, i, d, d]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def shape_props(rx, ry, rz, e1, e2):
    out = np.zeros(5)
    lib().sqo_shape_props(rx, ry, rz, e1, e2, _dp(out))
    return out


def surface(shape5, ph0, ph1):
    out = np.zeros(3)
    lib().sqo_surface(*[float(x) for x in shape5], ph0, ph1, _dp(out))
    return out


def normal(shape5, ph0, ph1):
    out = np.zeros(3)
    lib().sqo_normal(*[float(x) for x in shape5], ph0, ph1, _dp(out))
    return out


def curvatures(shape5, ph0, ph1):
    """Superquadrics::Curvatures of an unrotated shape: (k1, k2), dirMax, dirMin, maxFlag."""
    out = np.zeros(9)
    lib().sqo_curvatures(*[float(x) for x in shape5], float(ph0), float(ph1), _dp(out))
    return out[0:2], out[2:5], out[5:8], bool(out[8])


def hertz_mindlin(c1, c2, theta):
    """SuperquadricsGeom2::HertzMindlin: (curvatures_sum, alpha, K, E)."""
    a = np.ascontiguousarray(c1, dtype=np.float64)
    b = np.ascontiguousarray(c2, dtype=np.float64)
    out = np.zeros(4)
    lib().sqo_hertz_mindlin(_dp(a), _dp(b), float(theta), _dp(out))
    return tuple(out)


def disfunction(shapeA, qA, posA, shapeB, qB, posB, pa0, pa1, margins=False):
    """One FP64 Disfunction evaluation between two free superellipsoids: (p1, p2, stop_flag[,
    margins])."""
    out = np.zeros(7)
    m = np.zeros(10)
    a = [np.ascontiguousarray(x, dtype=np.float64) for x in (shapeA, qA, posA, shapeB, qB, posB)]
    lib().sqo_disfunction(*[_dp(x) for x in a], float(pa0), float(pa1), _dp(out), _dp(m) if margins else None)
    r = (out[0:3], out[3:6], bool(out[6]))
    return r + (m,) if margins else r


def lmder2(shapeA, qA, posA, shapeB, qB, posB, p0):
    """One lmder2 call: dict of the final angles, p1, p2, contact, touching, iterations, stop
    code and Disfunction evaluations."""
    out = np.zeros(15)
    a = [np.ascontiguousarray(x, dtype=np.float64) for x in (shapeA, qA, posA, shapeB, qB, posB, p0)]
    lib().sqo_lmder2(*[_dp(x) for x in a], _dp(out))
    return {"p": out[0:2], "p1": out[2:5], "p2": out[5:8], "contact": out[8:11], "touching": bool(out[11]),
            "iters": int(out[12]), "stop": int(out[13]), "evals": int(out[14])}


def normal2phi(shape5, n):
    out = np.zeros(2)
    n = np.ascontiguousarray(n, dtype=np.float64)
    lib().sqo_normal2phi(*[float(x) for x in shape5], _dp(n), _dp(out))
    return out


def set_math_noise(seed, rel=0.0):
    """Last-bit noise on the narrowphase's pow/sin/cos/atan2 results (seed 0: off).  rel = 0 moves
    a result by one ulp, rel > 0 by rel * |value|; the sign (-1, 0, +1) comes from a hash of the
    value and the seed.  Process-wide; set between steps."""
    lib().sqo_set_math_noise(int(seed), float(rel))


class OracleScene:
    """A reference-semantics scene on the CPU."""

    def __init__(self, threads=1):
        self.L = lib()
        self.h = self.L.sqo_create()
        self.L.sqo_set_threads(self.h, threads)

    def set_threads(self, n):
        self.L.sqo_set_threads(self.h, int(n))

    def close(self):
        if self.h:
            self.L.sqo_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @classmethod
    def from_spec(cls, spec, threads=1):
        o = cls(threads)
        m = spec.materials
        for k in range(len(m["Kn"])):
            o.L.sqo_add_material(o.h, m["Kn"][k], m["Ks"][k], m["frictionAngle"][k], m["betan"][k], m["betas"][k],
                                 m["density"][k])
        for i in range(spec.n_bodies):
            st = spec.state[i]
            pos = np.ascontiguousarray(st[0:3])
            if spec.kind[i] == 1:
                o.L.sqo_add_wall(o.h, _dp(pos), int(spec.wall_axis_sense[i, 0]), int(spec.wall_axis_sense[i, 1]),
                                 int(spec.mat[i]))
            else:
                q = np.ascontiguousarray(st[3:7])
                s = spec.shape5[i]
                o.L.sqo_add_sq(o.h, s[0], s[1], s[2], s[3], s[4], int(spec.mat[i]), _dp(q), int(spec.isSphere[i]),
                               _dp(pos))
        p = spec.params
        g = np.ascontiguousarray(p["gravity"], dtype=np.float64)
        o.L.sqo_set_params(o.h, p["dt"], _dp(g), p["damping"], p["verletDist"], int(p["targetInterv"]),
                           p["minSweepDistFactor"], int(p["sortAxis"]))
        o.n = spec.n_bodies
        if "G" in m:
            for k in range(len(m["G"])):
                o.L.sqo_set_moduli(o.h, k, float(m["G"][k]), float(m["nu"][k]))
        if spec.info.get("contact_model", "linear") == "hertz_mindlin":
            o.set_contact_model("hertz_mindlin")
        if spec.info.get("periodic"):
            o.set_periodic(spec.info["hSize"], spec.info.get("velGrad"))
        # velocities from the spec (the factory leaves them zero)
        if np.any(spec.state[:, 7:16] != 0):
            b = o.bodies()
            b[:, 7:16] = spec.state[:, 7:16]
            o.set_bodies(b)
        return o

    def set_periodic(self, hSize, velGrad=None):
        h = np.ascontiguousarray(hSize, dtype=np.float64).reshape(9)
        vg = None if velGrad is None else np.ascontiguousarray(velGrad, dtype=np.float64).reshape(9)
        self.L.sqo_set_periodic(self.h, _dp(h), _dp(vg) if vg is not None else None)

    def set_velgrad(self, velGrad):
        vg = np.ascontiguousarray(velGrad, dtype=np.float64).reshape(9)
        self.L.sqo_set_velgrad(self.h, _dp(vg))

    def cell(self):
        out = np.zeros(33)
        self.L.sqo_get_cell(self.h, _dp(out))
        return out

    def put_cell(self, c):
        c = np.ascontiguousarray(c, dtype=np.float64).reshape(33)
        self.L.sqo_set_cell(self.h, _dp(c))

    def step(self, n=1):
        self.L.sqo_step(self.h, int(n))

    def collide(self):
        return self.L.sqo_collide(self.h)

    def last_step_collided(self):
        return bool(self.L.sqo_last_step_collided(self.h))

    @property
    def iter(self):
        return self.L.sqo_iter(self.h)

    def bodies(self):
        n = self.L.sqo_num_bodies(self.h)
        out = np.zeros((n, BODY_STRIDE))
        self.L.sqo_get_bodies(self.h, _dp(out))
        return out

    def set_bodies(self, b):
        b = np.ascontiguousarray(b, dtype=np.float64)
        self.L.sqo_set_bodies(self.h, _dp(b))

    def interactions(self):
        n = self.L.sqo_num_interactions(self.h)
        out = np.zeros((max(n, 1), INTR_STRIDE))
        if n:
            self.L.sqo_get_interactions(self.h, _dp(out))
        return out[:n]

    def margins(self):
        """Decision margins of the last step, one row per interaction (order of interactions()):
        |c.(p2-p1)| (m), ||cos|-0.95|, |Dp-1e-5|/1e-5, |dF| (m), |J^T f - 1e-15|/1e-15, restart
        distance, isInside distance, |depth| (m), smallest ill-conditioned trig value,
        evaluations."""
        n = self.L.sqo_num_interactions(self.h)
        out = np.zeros((max(n, 1), 10))
        if n:
            self.L.sqo_get_margins(self.h, _dp(out))
        return out[:n]

    def set_interactions(self, recs):
        recs = np.ascontiguousarray(recs, dtype=np.float64).reshape(-1, INTR_STRIDE)
        self.L.sqo_set_interactions(self.h, len(recs), _dp(recs))

    def scalars(self):
        out = np.zeros(9)
        self.L.sqo_get_scalars(self.h, _dp(out))
        return out

    def set_scalars(self, s):
        s = np.ascontiguousarray(s, dtype=np.float64)
        self.L.sqo_set_scalars(self.h, _dp(s))

    def rebuild_sorted_bounds(self):
        self.L.sqo_rebuild_sorted_bounds(self.h)

    def stats(self):
        out = (C.c_long * 5)()
        self.L.sqo_stats(self.h, out)
        return dict(zip(("lm_calls", "lm_iterations", "dis_calls", "restarts", "nan_normals"), list(out)))

    def set_servo(self, config):
        cfg = np.ascontiguousarray(config, dtype=np.float64)
        assert cfg.shape == (30,)
        self.L.sqo_set_servo(self.h, _dp(cfg))

    def servo_state(self):
        out = np.zeros(36)
        self.L.sqo_get_servo(self.h, _dp(out))
        return out

    def put_servo(self, state):
        st = np.ascontiguousarray(state, dtype=np.float64)
        self.L.sqo_put_servo(self.h, _dp(st))

    def set_contact_model(self, model):
        self.L.sqo_set_contact_model(self.h, {"linear": 0, "hertz_mindlin": 1}[model])

    def set_moduli(self, mat, G, nu):
        self.L.sqo_set_moduli(self.h, int(mat), float(G), float(nu))

    def nan_forces(self):
        out = C.c_long(0)
        self.L.sqo_stats_nan_forces(self.h, C.byref(out))
        return out.value

    def pair_geom2(self, ia, ib, prior=None):
        out = np.zeros(25)
        pr = np.zeros(4) if prior is None else np.ascontiguousarray(prior, dtype=np.float64)
        it = self.L.sqo_pair_geom2(self.h, ia, ib, 1 if prior is None else 0, _dp(pr), _dp(out))
        return {"depth": out[0], "normal": out[1:4], "contactPoint": out[4:7], "point1": out[7:10],
                "point2": out[10:13], "contactAngle": out[13:15], "curvatures1": out[15:17],
                "curvatures2": out[17:19], "curvatureAngle": out[19], "alpha": out[20], "K": out[21], "E": out[22],
                "curvatures_sum": out[23], "isSphere": bool(out[24]), "nm_evaluations": it}

    def set_frozen(self, on=True):
        """Frozen-pair window: no collider pass, no bound-separation erase; signature reset."""
        self.L.sqo_set_frozen(self.h, 1 if on else 0)

    def signature(self):
        return int(self.L.sqo_signature(self.h))

    def reset_phys(self):
        self.L.sqo_reset_phys(self.h)

    def set_material(self, m, Kn, Ks, frictionAngle):
        self.L.sqo_set_material(self.h, int(m), float(Kn), float(Ks), float(frictionAngle))

    def set_eps(self, body, e1, e2):
        self.L.sqo_set_eps(self.h, int(body), float(e1), float(e2))

    def set_periodic_fix(self, on=True):
        """Fixture option (not the reference's behaviour): torque arm and relative velocity of
        contacts across the periodic boundary taken with the image shift."""
        self.L.sqo_set_periodic_fix(self.h, 1 if on else 0)

    def set_quiet(self, on=True):
        self.L.sqo_set_quiet(self.h, 1 if on else 0)

    def unbalanced_force(self, use_max=False):
        return float(self.L.sqo_unbalanced_force(self.h, 1 if use_max else 0))

    def get_stress(self, volume=0.0):
        out = np.zeros(9)
        self.L.sqo_get_stress(self.h, float(volume), _dp(out))
        return out.reshape(3, 3)

    def eval_hist(self):
        out = (C.c_long * 16)()
        self.L.sqo_eval_hist(self.h, out)
        return list(out)

    def pair_geom(self, ia, ib, prior=None):
        out = np.zeros(15)
        pr = np.zeros(4) if prior is None else np.ascontiguousarray(prior, dtype=np.float64)
        it = self.L.sqo_pair_geom(self.h, ia, ib, 1 if prior is None else 0, _dp(pr), _dp(out))
        return {"depth": out[0], "normal": out[1:4], "contactPoint": out[4:7], "point1": out[7:10],
                "point2": out[10:13], "contactAngle": out[13:15], "lm_iterations": it}
