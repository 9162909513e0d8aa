"""Gradients of a window of timesteps (the adjoint behind the C ABI's ``sqdem_adj_*``).

A window starts from a scene state and keeps its potential-pair set (no collider pass, no
bound-separation erase inside the window).  The loss is ``sum_b wF_b . F_b + wX_b . x_b``: the
contact force of each body in the window's last step (for a wall, the wall force) and the
final positions.  Parameters: per-body exponents ``eps`` (n x 2), per-material ``Kn``, ``Ks`` and
friction coefficient ``mu`` (the tangent of the reference's frictionAngle).  Ip2
(pkg/dem/Superquadrics.cpp:1086-1116) is applied afresh to every pair at the window's start.

:class:`AdjointWindow` is the plain interface; :func:`window_loss` wraps it as a
``torch.autograd.Function`` so that the loss is a differentiable torch scalar.  The gradient is
that of the discrete map with every branch taken as in the forward run; the forward run
returns a 64-bit signature of those branches.
"""
import ctypes as C
import math

import numpy as np

from . import _native
from ._native import BODY_STRIDE, INTR_STRIDE, SqdemError, _dp, _ip, load_library


def check_window_spec(spec):
    """Raise ValueError for a scene the adjoint window does not model: a periodic cell, viscous
    contact damping (betan/betas), the Hertz-Mindlin contact model, particles flagged as
    spheres."""
    if spec.info.get("periodic"):
        raise ValueError("the adjoint window has no periodic cell")
    if spec.info.get("contact_model", "linear") != "linear":
        raise ValueError("the adjoint window differentiates the linear contact model only")
    m = spec.materials
    if np.any(np.asarray(m["betan"]) > 1e-5) or np.any(np.asarray(m["betas"]) > 1e-5):
        raise ValueError("the adjoint window has no viscous contact damping (betan, betas must be 0)")
    if np.any((np.asarray(spec.kind) == 0) & (np.asarray(spec.isSphere) != 0)):
        raise ValueError("the adjoint window supports superquadrics not flagged as spheres")


class AdjointWindow:
    """One scene's window on one GPU (no CPU fallback: raises without a device)."""

    def __init__(self, device=0):
        self.lib = load_library()
        self.h = C.c_void_p()
        st = self.lib.sqdem_adj_create(C.byref(self.h), int(device))
        if st:
            self.h = None
            raise SqdemError(st, "sqdem_adj_create failed (no CUDA device?)")
        self.n = 0
        self.nmat = 0
        self.run_id = 0

    def _check(self, st):
        if st:
            raise SqdemError(st, self.lib.sqdem_adj_last_error(self.h).decode())

    def close(self):
        if self.h:
            self.lib.sqdem_adj_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def load(self, spec, state=None, interactions=None):
        """Window start: the bodies of ``spec`` (a SceneSpec) in ``state`` (n x 37, default the
        spec's), the interaction records ``interactions`` (m x 57, default none), the spec's
        dt, gravity and damping, its materials and exponents."""
        check_window_spec(spec)
        n = spec.n_bodies
        st = np.ascontiguousarray(spec.state if state is None else state, dtype=np.float64).reshape(n, BODY_STRIDE)
        recs = np.zeros((0, INTR_STRIDE)) if interactions is None else interactions
        recs = np.ascontiguousarray(recs, dtype=np.float64).reshape(-1, INTR_STRIDE)
        kind = np.ascontiguousarray(spec.kind, dtype=np.int32)
        shape5 = np.ascontiguousarray(spec.shape5, dtype=np.float64)
        was = np.ascontiguousarray(spec.wall_axis_sense, dtype=np.int32)
        mat = np.ascontiguousarray(spec.mat, dtype=np.int32)
        sph = np.ascontiguousarray(spec.isSphere, dtype=np.int32)
        g = np.ascontiguousarray(spec.params["gravity"], dtype=np.float64)
        self._check(self.lib.sqdem_adj_load(self.h, n, _ip(kind), _dp(shape5), _ip(was), _ip(mat), _ip(sph), _dp(st),
                                            len(recs), _dp(recs), float(spec.params["dt"]), _dp(g),
                                            float(spec.params["damping"])))
        self.n = n
        m = spec.materials
        self.set_materials(m["Kn"], m["Ks"], np.tan(np.asarray(m["frictionAngle"], dtype=np.float64)))
        self.set_eps(spec.shape5[:, 3:5])

    @classmethod
    def from_engine(cls, engine, spec, device=0):
        """A window starting from the current state of an Engine built from ``spec``."""
        w = cls(device)
        w.load(spec, engine.body_state(), engine.interactions(include_potential=True))
        return w

    def set_materials(self, Kn, Ks, mu):
        Kn, Ks, mu = (np.ascontiguousarray(x, dtype=np.float64).reshape(-1) for x in (Kn, Ks, mu))
        fa = np.arctan(mu)
        self._check(self.lib.sqdem_adj_set_materials(self.h, len(Kn), _dp(Kn), _dp(Ks), _dp(fa)))
        self.nmat = len(Kn)

    def set_eps(self, eps):
        e = np.ascontiguousarray(eps, dtype=np.float64).reshape(self.n, 2)
        self._check(self.lib.sqdem_adj_set_eps(self.h, _dp(e)))

    def forward(self, nsteps, checkpoint_every=100, wF=None, wX=None):
        """Run the window; returns (loss, branch signature)."""
        def w3(x):
            if x is None:
                return None
            return np.ascontiguousarray(x, dtype=np.float64).reshape(self.n, 3)
        a, b = w3(wF), w3(wX)
        loss = C.c_double()
        sig = C.c_ulonglong()
        self._check(self.lib.sqdem_adj_forward(self.h, int(nsteps), int(checkpoint_every),
                                               _dp(a) if a is not None else None, _dp(b) if b is not None else None,
                                               C.byref(loss), C.byref(sig)))
        self.run_id += 1
        return loss.value, sig.value

    def backward(self):
        """Gradient of the last forward run's loss: dict of eps (n x 2), Kn, Ks, mu."""
        ge = np.zeros((self.n, 2))
        gkn, gks, gmu = np.zeros(self.nmat), np.zeros(self.nmat), np.zeros(self.nmat)
        self._check(self.lib.sqdem_adj_backward(self.h, _dp(ge), _dp(gkn), _dp(gks), _dp(gmu)))
        return {"eps": ge, "Kn": gkn, "Ks": gks, "mu": gmu}

    def state(self):
        out = np.zeros((self.n, 16))
        self._check(self.lib.sqdem_adj_get_state(self.h, _dp(out)))
        return out

    REPLAY_SHAPES = {0: "1 lane x 17 tangents", 1: "3 lanes x 6", 2: "2 lanes x 9", 3: "6 lanes x 3"}

    def set_replay(self, shape=3):
        """Shape of the pairs' reverse-step kernel (REPLAY_SHAPES); the gradients are bitwise the
        same for every shape."""
        self._check(self.lib.sqdem_adj_set_replay(self.h, int(shape)))

    def set_replay_blocks(self, blocks_per_sm=1):
        """Resident blocks per SM of the grouped reverse-step kernels (0: unbounded); the
        gradients are bitwise the same for every value (see include/sqdem.h)."""
        self._check(self.lib.sqdem_adj_set_replay_blocks(self.h, int(blocks_per_sm)))

    BRANCH_NATURAL, BRANCH_RECORD, BRANCH_FORCE = 0, 1, 2

    def set_branches(self, mode):
        """Branch tape of the following forward runs: BRANCH_NATURAL evaluates every decision,
        BRANCH_RECORD records their outcomes, BRANCH_FORCE takes the recorded outcomes (a run
        with perturbed parameters then stays on the recorded branches; see include/sqdem.h)."""
        self._check(self.lib.sqdem_adj_set_branches(self.h, int(mode)))

    def branch_report(self):
        """Of the last forward run: decisions taken, forced decisions whose natural outcome
        differed, decisions beyond the tape (evaluated), steps recorded, and pair steps whose
        surface evaluations saw other signs of the local directions than the recorded run (a
        non-differentiable point of the superquadric surface crossed)."""
        out = np.zeros(5)
        self._check(self.lib.sqdem_adj_branch_report(self.h, _dp(out)))
        return dict(zip(("decisions", "disagreements", "unforced", "steps_recorded", "surface_sign_changes"),
                        out.astype(np.int64).tolist()))

    def set_forward(self, cooperative=True):
        """Forward kernel of the pairs: six lanes share each evaluation (default) or one thread
        per pair; the results are bitwise the same."""
        self._check(self.lib.sqdem_adj_set_forward(self.h, 1 if cooperative else 0))

    def num_pairs(self):
        return int(self.lib.sqdem_adj_num_pairs(self.h))

    def pairs(self):
        m = self.lib.sqdem_adj_num_pairs(self.h)
        out = np.zeros((max(m, 1), 16))
        self._check(self.lib.sqdem_adj_get_pairs(self.h, _dp(out)))
        return out[:m]

    def report(self):
        out = np.zeros(8)
        self._check(self.lib.sqdem_adj_report(self.h, _dp(out)))
        keys = ("replay_mismatches", "evaluations", "lm_calls", "pairs_replayed", "forward_ms", "backward_ms", "steps",
                "checkpoint_every")
        return dict(zip(keys, out.tolist()))


def _torch():
    import torch
    return torch


class _WindowLossFn:
    """Holder of the torch.autograd.Function (torch is imported lazily)."""
    fn = None

    @classmethod
    def get(cls):
        if cls.fn is not None:
            return cls.fn
        torch = _torch()

        class WindowLoss(torch.autograd.Function):
            @staticmethod
            def forward(ctx, eps, mu, Kn, Ks, window, nsteps, checkpoint_every, wF, wX):
                window.set_materials(Kn.detach().cpu().numpy(), Ks.detach().cpu().numpy(), mu.detach().cpu().numpy())
                window.set_eps(eps.detach().cpu().numpy())
                loss, sig = window.forward(nsteps, checkpoint_every, wF, wX)
                ctx.window = window
                ctx.run_id = window.run_id
                ctx.devs = (eps.device, mu.device, Kn.device, Ks.device)
                ctx.signature = sig
                return torch.tensor(loss, dtype=torch.float64, device=eps.device)

            @staticmethod
            def backward(ctx, g):
                w = ctx.window
                if w.run_id != ctx.run_id:
                    raise RuntimeError("the window ran again after this loss was computed; recompute the loss")
                gr = w.backward()
                s = float(g)
                t = lambda a, dev: torch.as_tensor(a * s, dtype=torch.float64, device=dev)  # noqa: E731
                return (t(gr["eps"], ctx.devs[0]), t(gr["mu"], ctx.devs[1]), t(gr["Kn"], ctx.devs[2]),
                        t(gr["Ks"], ctx.devs[3]), None, None, None, None, None)

        cls.fn = WindowLoss
        return WindowLoss


def window_loss(window, eps, mu, Kn, Ks, nsteps, checkpoint_every=100, wF=None, wX=None):
    """Differentiable loss of a window: torch float64 tensors eps (n x 2), mu, Kn, Ks (per
    material) -> scalar tensor; ``loss.backward()`` fills their ``.grad`` through the adjoint."""
    return _WindowLossFn.get().apply(eps, mu, Kn, Ks, window, int(nsteps), int(checkpoint_every), wF, wX)


def wall_force_weights(n, wall_id, axis, sign=1.0):
    """wF selecting one wall's force component (e.g. the top wall's normal force)."""
    w = np.zeros((n, 3))
    w[wall_id, axis] = sign
    return w


def tan_friction(spec):
    """Friction coefficients mu = tan(frictionAngle) of a spec's materials."""
    return np.array([math.tan(a) for a in spec.materials["frictionAngle"]])


__all__ = ["AdjointWindow", "check_window_spec", "window_loss", "wall_force_weights", "tan_friction"]
_ = _native
