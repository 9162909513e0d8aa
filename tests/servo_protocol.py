"""Config 2's servo-controlled specimen, the protocol of the long-run statistics
(tests/test_long_run_stats.py, tests/golden/make_compression_stats.py).

A closed cubic box of six walls around 500 superellipsoids on a 2.1 mm jittered lattice with the
walls against the outer particles (assemblies.config2's specimen, eps U[0.4, 1.6], friction 0.5,
kn = 1e5 N/m), run by config 2's CompressionEngine (pkg/dem/Compression.cpp:395-604): 100 kPa
held on the lateral walls, the top and bottom walls driven in strain (the shear phase of
action_cubic).  Recorded after DURATION seconds of simulated time (the number of steps follows
from the specimen's time step): the axial and mean lateral wall stresses, the porosity of the
box, the coordination number of the particles, the axial strain, and the mean penetration depth
of the touching particle pairs averaged over the last AVG_CHUNKS chunks (at a given stress it
scales as 1/kn: the contact stiffness's fingerprint).
"""
import numpy as np

from sudodem_gb300 import assemblies
from sudodem_gb300.servo import servo_config, state_dict

N = 500
DURATION = 0.035   # s of simulated time
CHUNK = 1000


def spec_and_config(seed, n=N, kn=1e5):
    spec = assemblies.cubic_specimen(n, seed=seed, friction=0.5, eps_range=(0.4, 1.6), spacing=2.1e-3, wall_gap=0.0,
                                     kn=kn)
    cfg = servo_config(z_servo=0, shearMode=1, goalx=1e5, goaly=1e5, goalz=0.05, max_vel=1.0, gain_alpha=0.5,
                       ramp_interval=200, ramp_chunks=20, echo_interval=1000, savedata_interval=1000,
                       target_strain=10.0)
    return spec, cfg


AVG_CHUNKS = 10   # chunks at the end over which the mean penetration depth is averaged


def _mean_depth(spec, recs):
    kind = spec.kind
    touching = (recs[:, 2] != 0) & (recs[:, 4] > 0)
    pp = touching & (kind[recs[:, 0].astype(int)] == 0) & (kind[recs[:, 1].astype(int)] == 0)
    return (float(np.mean(recs[pp, 4])) if np.any(pp) else 0.0), pp


class Run:
    """One specimen, advanced chunk by chunk (engine-agnostic: the oracle scene or the GPU engine,
    both with step, set_servo, servo_state and interactions)."""

    def __init__(self, spec, engine, cfg):
        self.spec, self.e = spec, engine
        engine.set_servo(cfg)
        self.steps = 0
        self.total = int(np.ceil(DURATION / spec.params["dt"]))
        self.done = False
        self.result = None
        self.depths = []

    def advance(self):
        n = min(CHUNK, self.total - self.steps)
        self.e.step(n)
        self.steps += n

    def check(self):
        if self.steps >= self.total - AVG_CHUNKS * CHUNK:
            self.depths.append(_mean_depth(self.spec, self.e.interactions())[0])
        if self.steps < self.total:
            return False
        self.done = True
        st = state_dict(self.e.servo_state())
        recs = self.e.interactions()
        _, pp = _mean_depth(self.spec, recs)
        self.result = {"axial_stress": st["wszz"], "lateral_stress": 0.5 * (st["wsxx"] + st["wsyy"]),
                       "porosity": 1.0 - st["particlesVolume"] / st["Current_boxVolume"],
                       "coordination": 2.0 * float(np.sum(pp)) / self.spec.n_particles, "axial_strain": st["strain2"],
                       "unbalanced_force": st["UnbalancedForce"], "mean_depth": float(np.mean(self.depths))}
        return True
