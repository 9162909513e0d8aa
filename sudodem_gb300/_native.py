"""ctypes binding of libsqdem_gpu.so (the C ABI declared in include/sqdem.h).

There is no CPU fallback: if the library cannot be loaded or no CUDA device is present,
the constructor raises.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build
from .shapes import BODY_STRIDE, INTR_STRIDE  # noqa: F401
NSCALARS = 9

SQDEM_SUPERQUADRIC = 0
SQDEM_WALL = 1
PRECISION = {"fp64": 0, "mixed": 1}

STATUS = {0: "OK", 1: "ERR_ARG", 2: "ERR_CUDA", 3: "ERR_CAPACITY", 4: "ERR_STATE", 5: "ERR_NUMERIC"}


class SqdemError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"sqdem {STATUS.get(status, status)}: {msg}")
        self.status = status


class _Tune(C.Structure):
    _fields_ = [("search", C.c_int), ("pass1", C.c_int), ("ms", C.c_double), ("n", C.c_int)]


class _Config(C.Structure):
    _fields_ = [("device", C.c_int), ("precision", C.c_int), ("contacts_per_body", C.c_int), ("use_graph", C.c_int)]


class _Params(C.Structure):
    _fields_ = [
        ("dt", C.c_double), ("gravity", C.c_double * 3), ("damping", C.c_double), ("verletDist", C.c_double),
        ("targetInterv", C.c_int), ("minSweepDistFactor", C.c_double), ("sortAxis", C.c_int),
        ("isSuperquadrics", C.c_int), ("exactAsphericalRot", C.c_int),
    ]


class _Report(C.Structure):
    _fields_ = [(n, C.c_longlong) for n in ("nan_normals", "nan_forces", "lm_calls", "lm_iterations", "lm_maxiter",
                                             "overflow", "collider_runs", "steps", "evals_fp32", "evals_fp64",
                                             "lm_rounds_max", "fallback_fp64", "lm_rounds_max_ff", "long_queue")]


_LIB = None


def library_path():
    return _build.LIB


def load_library(build_if_missing=True):
    """Load libsqdem_gpu.so from the package directory (building it if it is missing)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise OSError(f"{path} is missing; run sudodem_gb300.build.build()")
        _build.build()
    lib = C.CDLL(path)
    P = C.POINTER
    d, i, l, v = C.c_double, C.c_int, C.c_long, C.c_void_p
    dp, ip = P(d), P(i)
    sig = {
        "sqdem_create": (i, [P(v), P(_Config)]),
        "sqdem_destroy": (None, [v]),
        "sqdem_last_error": (C.c_char_p, [v]),
        "sqdem_set_materials": (i, [v, i, dp, dp, dp, dp, dp, dp]),
        "sqdem_set_bodies": (i, [v, i, ip, dp, ip, ip, ip, dp]),
        "sqdem_set_params": (i, [v, P(_Params)]),
        "sqdem_step": (i, [v, i]),
        "sqdem_sync": (i, [v, P(_Report)]),
        "sqdem_get_body_state": (i, [v, dp]),
        "sqdem_put_body_state": (i, [v, dp]),
        "sqdem_get_kinematics": (i, [v, dp]),
        "sqdem_put_kinematics": (i, [v, dp]),
        "sqdem_num_interactions": (i, [v, i, P(l)]),
        "sqdem_get_interactions": (i, [v, i, dp, l, P(l)]),
        "sqdem_put_interactions": (i, [v, l, dp]),
        "sqdem_get_scalars": (i, [v, dp]),
        "sqdem_put_scalars": (i, [v, dp]),
        "sqdem_stage_times": (i, [v, dp]),
        "sqdem_shape_props": (i, [d, d, d, d, d, dp]),
        "sqdem_launch_count": (C.c_longlong, [v]),
        "sqdem_set_record_full": (i, [v, i]),
        "sqdem_time_steps": (i, [v, i, dp]),
        "sqdem_time_e2e": (i, [v, i, v, v, dp]),
        "sqdem_time_contacts": (i, [v, i, dp]),
        "sqdem_set_use_graph": (i, [v, i]),
        "sqdem_set_lm_spread": (i, [v, i]), "sqdem_set_periodic_fix": (i, [v, i]),
        "sqdem_set_servo": (i, [v, dp]), "sqdem_get_servo": (i, [v, dp]), "sqdem_put_servo": (i, [v, dp]),
        "sqdem_set_quiet": (i, [v, i]), "sqdem_unbalanced_force": (i, [v, i, dp]),
        "sqdem_get_stress": (i, [v, C.c_double, dp]),
        "sqdem_batch_create": (i, [C.POINTER(v), i, C.c_void_p]), "sqdem_batch_destroy": (None, [v]),
        "sqdem_batch_last_error": (C.c_char_p, [v]), "sqdem_batch_size": (i, [v]),
        "sqdem_batch_scene": (i, [v, i, C.POINTER(v)]), "sqdem_batch_step": (i, [v, i]),
        "sqdem_batch_sync": (i, [v, C.c_void_p]), "sqdem_batch_time_steps": (i, [v, i, dp]),
        "sqdem_batch_time_e2e": (i, [v, i, C.c_void_p, C.c_void_p, dp]),
        "sqdem_batch_launch_count": (C.c_longlong, [v]),
        "sqdem_snapshot": (i, [v, C.c_void_p, C.POINTER(C.c_size_t)]), "sqdem_restore": (i, [v, C.c_void_p, C.c_size_t]),
        "sqdem_set_periodic": (i, [v, dp, dp]),
        "sqdem_set_velgrad": (i, [v, dp]),
        "sqdem_get_cell": (i, [v, dp]),
        "sqdem_put_cell": (i, [v, dp]),
        "sqdem_contacts_static_queue": (i, [v]),
        "sqdem_pipe_peaks": (i, [i, dp]),
        "sqdem_search_times": (i, [v, dp]),
        "sqdem_set_contact_model": (i, [v, i]), "sqdem_contact_model": (i, [v]), "sqdem_num_materials": (i, [v]),
        "sqdem_set_material_moduli": (i, [v, i, dp, dp]), "sqdem_get_material_moduli": (i, [v, dp, dp]),
        "sqdem_set_launch_shape": (i, [v, i, i]), "sqdem_autotune": (i, [v, i, C.c_void_p]),
        "sqdem_adj_create": (i, [P(v), i]), "sqdem_adj_destroy": (None, [v]),
        "sqdem_adj_last_error": (C.c_char_p, [v]),
        "sqdem_adj_load": (i, [v, i, ip, dp, ip, ip, ip, dp, l, dp, d, dp, d]),
        "sqdem_adj_set_materials": (i, [v, i, dp, dp, dp]), "sqdem_adj_set_eps": (i, [v, dp]),
        "sqdem_adj_forward": (i, [v, i, i, dp, dp, dp, P(C.c_ulonglong)]),
        "sqdem_adj_backward": (i, [v, dp, dp, dp, dp]), "sqdem_adj_get_state": (i, [v, dp]),
        "sqdem_adj_num_pairs": (l, [v]), "sqdem_adj_get_pairs": (i, [v, dp]), "sqdem_adj_report": (i, [v, dp]),
        "sqdem_adj_set_replay": (i, [v, i]), "sqdem_adj_set_forward": (i, [v, i]),
        "sqdem_adj_set_replay_blocks": (i, [v, i]), "sqdem_adj_set_branches": (i, [v, i]),
        "sqdem_adj_branch_report": (i, [v, dp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _LIB = lib
    return lib


def exported_symbols():
    return ["sqdem_create", "sqdem_destroy", "sqdem_last_error", "sqdem_set_materials", "sqdem_set_bodies",
            "sqdem_set_params", "sqdem_step", "sqdem_sync", "sqdem_get_body_state", "sqdem_put_body_state",
            "sqdem_get_kinematics", "sqdem_put_kinematics", "sqdem_num_interactions", "sqdem_get_interactions",
            "sqdem_put_interactions", "sqdem_get_scalars", "sqdem_put_scalars", "sqdem_stage_times",
            "sqdem_shape_props", "sqdem_launch_count", "sqdem_set_record_full", "sqdem_time_steps",
            "sqdem_time_e2e", "sqdem_time_contacts", "sqdem_set_use_graph", "sqdem_set_lm_spread", "sqdem_set_periodic_fix", "sqdem_set_periodic",
            "sqdem_set_velgrad", "sqdem_get_cell", "sqdem_put_cell", "sqdem_contacts_static_queue", "sqdem_pipe_peaks", "sqdem_search_times",
            "sqdem_set_servo", "sqdem_get_servo", "sqdem_put_servo", "sqdem_set_quiet", "sqdem_unbalanced_force",
            "sqdem_get_stress", "sqdem_batch_create", "sqdem_batch_destroy", "sqdem_batch_last_error",
            "sqdem_batch_size", "sqdem_batch_scene", "sqdem_batch_step", "sqdem_batch_sync", "sqdem_batch_time_steps",
            "sqdem_batch_time_e2e", "sqdem_batch_launch_count", "sqdem_snapshot", "sqdem_restore",
            "sqdem_set_contact_model", "sqdem_contact_model", "sqdem_num_materials", "sqdem_set_material_moduli",
            "sqdem_get_material_moduli", "sqdem_set_launch_shape", "sqdem_autotune",
            "sqdem_adj_create", "sqdem_adj_destroy", "sqdem_adj_last_error", "sqdem_adj_load",
            "sqdem_adj_set_materials", "sqdem_adj_set_eps", "sqdem_adj_forward", "sqdem_adj_backward",
            "sqdem_adj_get_state", "sqdem_adj_num_pairs", "sqdem_adj_get_pairs", "sqdem_adj_report",
            "sqdem_adj_set_replay", "sqdem_adj_set_forward", "sqdem_adj_set_replay_blocks", "sqdem_adj_set_branches",
            "sqdem_adj_branch_report"]


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def pipe_peaks(device=0):
    """Measured pipe peaks of the GPU: FP64 and FP32 FMA TFLOP/s and the FP64 and double-float
    Disfunction evaluation rates (1e9/s) of a saturated grid (sqdem_pipe_peaks)."""
    lib = load_library()
    out = np.zeros(4)
    st = lib.sqdem_pipe_peaks(int(device), _dp(out))
    if st:
        raise SqdemError(st, "sqdem_pipe_peaks failed")
    return {"fp64_tflops": out[0], "fp32_tflops": out[1], "disfunction_fp64_geval_s": out[2],
            "disfunction_ff_geval_s": out[3]}


def shape_props(rx, ry, rz, eps1, eps2):
    """Superquadrics::Initial: (volume, Ixx, Iyy, Izz, r_max) at unit density."""
    lib = load_library()
    out = np.zeros(5)
    st = lib.sqdem_shape_props(rx, ry, rz, eps1, eps2, _dp(out))
    if st:
        raise SqdemError(st, "bad shape parameters")
    return out


class Engine:
    """One GPU scene behind the C ABI."""

    def __init__(self, device=0, precision="fp64", contacts_per_body=16, use_graph=True, _handle=None):
        self.lib = load_library()
        self.n = 0
        if _handle is not None:     # a scene of a Batch: the batch owns the context
            self.h, self._owned = _handle, False
            return
        self._owned = True
        self.h = C.c_void_p()
        cfg = _Config(device, PRECISION[precision], contacts_per_body, 1 if use_graph else 0)
        st = self.lib.sqdem_create(C.byref(self.h), C.byref(cfg))
        if st:
            msg = self.lib.sqdem_last_error(self.h).decode()
            self.lib.sqdem_destroy(self.h)
            self.h = None
            raise SqdemError(st, msg)
        self.n = 0

    def _check(self, st):
        if st:
            raise SqdemError(st, self.lib.sqdem_last_error(self.h).decode())

    def close(self):
        if self.h and self._owned:
            self.lib.sqdem_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- set-up ---------------------------------------------------------------------------
    def set_materials(self, Kn, Ks, frictionAngle, betan, betas, density):
        arrs = [np.ascontiguousarray(x, dtype=np.float64) for x in (Kn, Ks, frictionAngle, betan, betas, density)]
        self._check(self.lib.sqdem_set_materials(self.h, len(arrs[0]), *[_dp(a) for a in arrs]))

    def set_bodies(self, kind, shape5, wall_axis_sense, mat, isSphere, state):
        kind = np.ascontiguousarray(kind, dtype=np.int32)
        n = len(kind)
        shape5 = np.ascontiguousarray(shape5, dtype=np.float64).reshape(n, 5)
        was = np.ascontiguousarray(wall_axis_sense, dtype=np.int32).reshape(n, 2)
        mat = np.ascontiguousarray(mat, dtype=np.int32)
        sph = np.ascontiguousarray(isSphere, dtype=np.int32)
        state = np.ascontiguousarray(state, dtype=np.float64).reshape(n, BODY_STRIDE)
        self._check(self.lib.sqdem_set_bodies(self.h, n, _ip(kind), _dp(shape5), _ip(was), _ip(mat), _ip(sph), _dp(state)))
        self.n = n

    def set_params(self, dt, gravity, damping, verletDist, targetInterv=50, minSweepDistFactor=0.1, sortAxis=0,
                   isSuperquadrics=1, exactAsphericalRot=1):
        p = _Params(dt, (C.c_double * 3)(*gravity), damping, verletDist, int(targetInterv), minSweepDistFactor,
                    int(sortAxis), int(isSuperquadrics), int(exactAsphericalRot))
        self._check(self.lib.sqdem_set_params(self.h, C.byref(p)))

    def load(self, spec):
        """Load a scene description (see sudodem_gb300.assemblies.SceneSpec)."""
        m = spec.materials
        self.set_materials(m["Kn"], m["Ks"], m["frictionAngle"], m["betan"], m["betas"], m["density"])
        self.set_params(**spec.params)
        if "G" in m:
            self.set_material_moduli(m["G"], m["nu"])
        self.set_bodies(spec.kind, spec.shape5, spec.wall_axis_sense, spec.mat, spec.isSphere, spec.state)
        if spec.info.get("periodic"):
            self.set_periodic(spec.info["hSize"], spec.info.get("velGrad"))
        self.set_contact_model(spec.info.get("contact_model", "linear"))

    def set_use_graph(self, on=True):
        self._check(self.lib.sqdem_set_use_graph(self.h, 1 if on else 0))

    def set_lm_spread(self, on=True):
        self._check(self.lib.sqdem_set_lm_spread(self.h, 1 if on else 0))

    def set_periodic_fix(self, on=True):
        """Periodic-boundary correction (off by default, the reference's behaviour): see
        sqdem_set_periodic_fix in include/sqdem.h."""
        self._check(self.lib.sqdem_set_periodic_fix(self.h, 1 if on else 0))

    def set_launch_shape(self, search_blocks_per_sm=0, pass1_blocks_per_sm=0):
        """Launch shapes of the contact stage (0 keeps the default); results are unchanged."""
        self._check(self.lib.sqdem_set_launch_shape(self.h, int(search_blocks_per_sm), int(pass1_blocks_per_sm)))

    def autotune(self, steps=5):
        """Time the candidate launch shapes on this scene and keep the fastest.  The tuning
        steps are ordinary timesteps (launch shapes change no result): the scene advances."""
        t = _Tune()
        self._check(self.lib.sqdem_autotune(self.h, int(steps), C.byref(t)))
        return {"search_blocks_per_sm": t.search, "pass1_blocks_per_sm": t.pass1, "ms_per_step": t.ms,
                "candidates": t.n}

    CONTACT_MODELS = {"linear": 0, "hertz_mindlin": 1}

    def set_contact_model(self, model):
        """'linear' (SuperquadricsGeom/Phys/Law) or 'hertz_mindlin' (SuperquadricsGeom2,
        HertzMindlinPhys, SuperquadricsLaw2)."""
        if model not in self.CONTACT_MODELS:
            raise ValueError("contact model must be 'linear' or 'hertz_mindlin'")
        self._check(self.lib.sqdem_set_contact_model(self.h, self.CONTACT_MODELS[model]))

    def contact_model(self):
        k = self.lib.sqdem_contact_model(self.h)
        return {v: n for n, v in self.CONTACT_MODELS.items()}[k]

    def set_material_moduli(self, G, nu):
        """SuperquadricsMat2 shear modulus G and Poisson's ratio nu per material."""
        G = np.ascontiguousarray(G, dtype=np.float64)
        nu = np.ascontiguousarray(nu, dtype=np.float64)
        if G.shape != nu.shape or G.ndim != 1:
            raise ValueError("G and nu must be 1-D arrays of the same length")
        self._check(self.lib.sqdem_set_material_moduli(self.h, len(G), _dp(G), _dp(nu)))

    def material_moduli(self):
        n = self.lib.sqdem_num_materials(self.h)
        G, nu = np.zeros(n), np.zeros(n)
        self._check(self.lib.sqdem_get_material_moduli(self.h, _dp(G), _dp(nu)))
        return G, nu

    # CompressionEngine, quiet flag, Shop reductions
    def set_servo(self, config):
        from .servo import CONFIG_SIZE
        cfg = np.ascontiguousarray(config, dtype=np.float64)
        assert cfg.shape == (CONFIG_SIZE,)
        self._check(self.lib.sqdem_set_servo(self.h, _dp(cfg)))

    def servo_state(self):
        from .servo import STATE_SIZE
        out = np.zeros(STATE_SIZE)
        self._check(self.lib.sqdem_get_servo(self.h, _dp(out)))
        return out

    def put_servo(self, state):
        st = np.ascontiguousarray(state, dtype=np.float64)
        self._check(self.lib.sqdem_put_servo(self.h, _dp(st)))

    def snapshot(self):
        """The whole state as bytes (sqdem_snapshot); restore() continues bit for bit from it."""
        size = C.c_size_t(0)
        self._check(self.lib.sqdem_snapshot(self.h, None, C.byref(size)))
        buf = C.create_string_buffer(size.value)
        self._check(self.lib.sqdem_snapshot(self.h, C.cast(buf, C.c_void_p), C.byref(size)))
        return buf.raw[:size.value]

    def restore(self, blob):
        buf = C.create_string_buffer(blob, len(blob))
        self._check(self.lib.sqdem_restore(self.h, C.cast(buf, C.c_void_p), len(blob)))
        self.n = int(np.frombuffer(blob[32:40], dtype=np.int64)[0])   # SnapHeader.N

    def set_quiet(self, on=True):
        self._check(self.lib.sqdem_set_quiet(self.h, 1 if on else 0))

    def unbalanced_force(self, use_max=False):
        out = np.zeros(1)
        self._check(self.lib.sqdem_unbalanced_force(self.h, 1 if use_max else 0, _dp(out)))
        return float(out[0])

    def get_stress(self, volume=0.0):
        out = np.zeros(9)
        self._check(self.lib.sqdem_get_stress(self.h, float(volume), _dp(out)))
        return out.reshape(3, 3)

    def set_record_full(self, on=True):
        self._check(self.lib.sqdem_set_record_full(self.h, 1 if on else 0))

    # -- stepping -------------------------------------------------------------------------
    def step(self, n=1):
        self._check(self.lib.sqdem_step(self.h, int(n)))

    def sync(self):
        r = _Report()
        st = self.lib.sqdem_sync(self.h, C.byref(r))
        rep = {f: getattr(r, f) for f, _ in _Report._fields_}
        self._check(st)
        return rep

    def stage_times(self):
        out = np.zeros(3)
        self._check(self.lib.sqdem_stage_times(self.h, _dp(out)))
        return out

    def search_times(self):
        """(search kernel ms, FP64 fallback kernel ms) summed over the last eager step() call."""
        out = np.zeros(2)
        self._check(self.lib.sqdem_search_times(self.h, _dp(out)))
        return out

    def time_steps(self, n):
        """Device milliseconds of n timesteps (events on the engine stream)."""
        ms = C.c_double()
        self._check(self.lib.sqdem_time_steps(self.h, int(n), C.byref(ms)))
        return ms.value

    def time_e2e(self, n, in_ptr, out_ptr):
        """Device milliseconds of n x (H2D kinematics, step, D2H kinematics); pointers to host
        buffers of 16 doubles per body (pinned for asynchronous copies)."""
        ms = C.c_double()
        self._check(self.lib.sqdem_time_e2e(self.h, int(n), C.c_void_p(in_ptr), C.c_void_p(out_ptr), C.byref(ms)))
        return ms.value

    def time_contacts(self, nrep=1):
        ms = C.c_double()
        self._check(self.lib.sqdem_time_contacts(self.h, int(nrep), C.byref(ms)))
        return ms.value

    def contacts_static_queue(self):
        """One contact-stage pass with the work queue in the library's static device array
        (no allocation; see include/sqdem.h)."""
        self._check(self.lib.sqdem_contacts_static_queue(self.h))

    def launch_count(self):
        return int(self.lib.sqdem_launch_count(self.h))

    # -- state exchange -------------------------------------------------------------------
    def body_state(self):
        out = np.zeros((self.n, BODY_STRIDE))
        self._check(self.lib.sqdem_get_body_state(self.h, _dp(out)))
        return out

    def put_body_state(self, st):
        st = np.ascontiguousarray(st, dtype=np.float64).reshape(self.n, BODY_STRIDE)
        self._check(self.lib.sqdem_put_body_state(self.h, _dp(st)))

    def kinematics(self, out=None):
        if out is None:
            out = np.zeros((self.n, 16))
        self._check(self.lib.sqdem_get_kinematics(self.h, _dp(out)))
        return out

    def put_kinematics(self, k):
        k = np.ascontiguousarray(k, dtype=np.float64).reshape(self.n, 16)
        self._check(self.lib.sqdem_put_kinematics(self.h, _dp(k)))

    def interactions(self, include_potential=True):
        n = C.c_long()
        self._check(self.lib.sqdem_num_interactions(self.h, 1 if include_potential else 0, C.byref(n)))
        out = np.zeros((max(n.value, 1), INTR_STRIDE))
        got = C.c_long()
        self._check(self.lib.sqdem_get_interactions(self.h, 1 if include_potential else 0, _dp(out), n.value,
                                                    C.byref(got)))
        return out[: got.value]

    def put_interactions(self, recs):
        recs = np.ascontiguousarray(recs, dtype=np.float64).reshape(-1, INTR_STRIDE)
        self._check(self.lib.sqdem_put_interactions(self.h, len(recs), _dp(recs)))

    def set_periodic(self, hSize, velGrad=None):
        h = np.ascontiguousarray(hSize, dtype=np.float64).reshape(9)
        vg = None if velGrad is None else np.ascontiguousarray(velGrad, dtype=np.float64).reshape(9)
        self._check(self.lib.sqdem_set_periodic(self.h, _dp(h), _dp(vg) if vg is not None else None))

    def set_velgrad(self, velGrad):
        vg = np.ascontiguousarray(velGrad, dtype=np.float64).reshape(9)
        self._check(self.lib.sqdem_set_velgrad(self.h, _dp(vg)))

    def cell(self):
        out = np.zeros(33)
        self._check(self.lib.sqdem_get_cell(self.h, _dp(out)))
        return out

    def put_cell(self, c):
        c = np.ascontiguousarray(c, dtype=np.float64).reshape(33)
        self._check(self.lib.sqdem_put_cell(self.h, _dp(c)))

    def scalars(self):
        out = np.zeros(NSCALARS)
        self._check(self.lib.sqdem_get_scalars(self.h, _dp(out)))
        return out

    def put_scalars(self, s):
        s = np.ascontiguousarray(s, dtype=np.float64)
        self._check(self.lib.sqdem_put_scalars(self.h, _dp(s)))


class Batch:
    """Independent specimens stepped together: one context per scene (``scenes[i]``, an
    Engine), one CUDA graph launch per step running every scene's step as a parallel branch."""

    def __init__(self, n_scenes, device=0, precision="fp64", contacts_per_body=16):
        self.lib = load_library()
        self.h = C.c_void_p()
        cfg = _Config(device, PRECISION[precision], contacts_per_body, 1)
        st = self.lib.sqdem_batch_create(C.byref(self.h), int(n_scenes), C.c_void_p(C.addressof(cfg)))
        if st:
            msg = self.lib.sqdem_batch_last_error(self.h).decode()
            self.lib.sqdem_batch_destroy(self.h)
            self.h = None
            raise SqdemError(st, msg)
        self.scenes = []
        for i in range(n_scenes):
            ctx = C.c_void_p()
            self._check(self.lib.sqdem_batch_scene(self.h, i, C.byref(ctx)))
            self.scenes.append(Engine(_handle=ctx))

    def _check(self, st):
        if st:
            raise SqdemError(st, self.lib.sqdem_batch_last_error(self.h).decode())

    def close(self):
        if self.h:
            for e in self.scenes:
                e.h = None
            self.lib.sqdem_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def load(self, specs, servo=None):
        for e, spec in zip(self.scenes, specs):
            e.load(spec)
            if servo is not None:
                e.set_servo(servo)

    @property
    def n_bodies(self):
        return sum(e.n for e in self.scenes)

    def step(self, n=1):
        self._check(self.lib.sqdem_batch_step(self.h, int(n)))

    def sync(self):
        r = _Report()
        st = self.lib.sqdem_batch_sync(self.h, C.c_void_p(C.addressof(r)))
        rep = {f: getattr(r, f) for f, _ in _Report._fields_}
        self._check(st)
        return rep

    def time_steps(self, n):
        ms = np.zeros(1)
        self._check(self.lib.sqdem_batch_time_steps(self.h, int(n), _dp(ms)))
        return float(ms[0])

    def time_e2e(self, n, in_ptr, out_ptr):
        ms = np.zeros(1)
        self._check(self.lib.sqdem_batch_time_e2e(self.h, int(n), C.c_void_p(in_ptr), C.c_void_p(out_ptr), _dp(ms)))
        return float(ms[0])

    def launch_count(self):
        return int(self.lib.sqdem_batch_launch_count(self.h))
