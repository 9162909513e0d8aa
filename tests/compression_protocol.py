"""Config 1's isotropic periodic compression to 100 kPa, the protocol of the long-run
statistics (tests/test_long_run_stats.py, tests/golden/make_compression_stats.py).

A periodic cube of superellipsoids (half-axes U[0.8,1.2] mm, eps1/eps2 U[0.3,1.8], uniform
random orientations, kn = 1e5 N/m, ks/kn = 0.5, friction 0.5, density 2650, local damping 0.3;
assemblies.periodic_cell) starts on a jittered lattice loose enough that no two bounding spheres
overlap, and is compressed by velGrad = -rate * I: 10/s through the gas phase until the mean
stress -tr(sigma)/3 of Shop::getStress (pkg/dem/Shop_02.cpp:350-376) reaches 1 kPa, then at
config 1's 1/s until it has reached 100 kPa at two checks CHUNK steps apart.  Both engines run
with the periodic-boundary correction on: with the reference's own torque arm and relative
velocity at the boundary (Superquadrics.cpp:1042-1045,1356) boundary particles spin up without
bound under compression, and the packing's statistics are then those of that instability.

Recorded per run: the steps to 1 kPa and to 100 kPa, and at 100 kPa the solid fraction, the
mean stress, the deviatoric stress (von Mises of sigma) and the coordination number (touching
particle-particle contacts per particle, cf. py/utils.py:498); then the packing's bulk
stiffness, the rise of the mean stress over a further volumetric strain of PROBE_STRAIN at the
same rate divided by that strain, which scales with the contact stiffness (a 30% stiffer or
stiffer-reporting contact law shows as a 30% higher value).
"""
import numpy as np

from sudodem_gb300 import assemblies

N = 2000
CHUNK = 500
GAS_RATE, SLOW_RATE = 10.0, 1.0
P_SWITCH, P_TARGET = 1e3, 1e5
MAX_STEPS = 600_000
PROBE_STRAIN = 3e-3   # volumetric strain of the stiffness probe after 100 kPa


def spec_for(seed, n=N, kn=1e5):
    probe = assemblies.periodic_cell(n, seed=seed, solid_fraction=0.3, eps_range=(0.3, 1.8), kn=kn)
    rmax = max(assemblies.shape_props(*probe.shape5[p])[4] for p in range(n))
    m = int(np.ceil(n ** (1.0 / 3.0)))
    vol = float(np.sum(probe.state[:, 33] / 2650.0))
    spacing = 2.0 * rmax / 0.9 * 1.01          # lattice gap above the largest bounding diameter
    phi0 = vol / (m * spacing) ** 3
    spec = assemblies.periodic_cell(n, seed=seed, solid_fraction=phi0, eps_range=(0.3, 1.8), strain_rate=GAS_RATE,
                                    kn=kn)
    spec.info["volume"] = vol
    return spec


def coordination(recs, n_particles):
    touching = (recs[:, 2] != 0) & (recs[:, 4] > 0)
    return 2.0 * np.sum(touching) / n_particles


class Run:
    """One compression, advanced chunk by chunk (engine-agnostic: the oracle scene or the GPU
    engine, both with step, get_stress, cell, set_velgrad, interactions)."""

    def __init__(self, spec, engine):
        self.spec, self.e = spec, engine
        self.vol = spec.info["volume"]
        self.steps = 0
        self.slow = False
        self.held = 0
        self.done = False
        self.at_switch = None
        self.result = None
        self.probe_steps = 0

    def check(self):
        """After a chunk: read the stress, switch rates, detect the end."""
        s = self.e.get_stress()
        p = -np.trace(s) / 3.0
        if not self.slow and p >= P_SWITCH:
            self.e.set_velgrad((-SLOW_RATE * np.eye(3)).reshape(9))
            self.slow = True
            self.at_switch = self.steps
        if self.result is not None:      # the stiffness probe has run
            dt = self.spec.params["dt"]
            eps_v = 3.0 * SLOW_RATE * self.probe_steps * dt
            self.result["bulk_stiffness"] = float((p - self.result["mean_stress"]) / eps_v)
            self.done = True
            return True
        self.held = self.held + 1 if p >= P_TARGET else 0
        if self.held >= 2 or self.steps >= MAX_STEPS:
            L = self.e.cell()[0:9].reshape(3, 3)
            dev = s - np.eye(3) * np.trace(s) / 3.0
            self.result = {"steps_to_1kPa": self.at_switch, "steps_to_100kPa": self.steps,
                           "solid_fraction": self.vol / abs(np.linalg.det(L)), "mean_stress": float(p),
                           "deviatoric_stress": float(np.sqrt(1.5 * np.sum(dev * dev))),
                           "coordination": float(coordination(self.e.interactions(), self.spec.n_particles)),
                           "reached": bool(self.held >= 2)}
            self.probe_steps = int(np.ceil(PROBE_STRAIN / (3.0 * SLOW_RATE * self.spec.params["dt"])))
        return False

    def advance(self):
        """Queue the next chunk (asynchronous on the GPU engine); after 100 kPa, the probe."""
        n = self.probe_steps if self.result is not None else CHUNK
        self.e.step(n)
        self.steps += n
