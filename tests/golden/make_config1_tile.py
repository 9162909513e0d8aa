"""Make tests/golden/config1_tile.npz: one periodic cell of config 1's particles compressed to
100 kPa mean stress, the tile of the dense config-1 workload (assemblies.config1_dense).

1,600 superellipsoids (half-axes U[0.8,1.2] mm, eps1/eps2 U[0.3,1.8], uniform random
orientations, kn = 1e5 N/m, ks/kn = 0.5, friction 0.5, density 2650, local damping 0.3) on a
jittered lattice in a periodic cube (assemblies.periodic_cell) loose enough that no two bounding
spheres overlap (config 1's own start at solid fraction 0.3 has lattice overlaps of up to
~0.1 mm, which throw particles at m/s and keep a hot, colliding gas whose collision stress is
not that of a jammed packing).  The CPU oracle compresses it isotropically (strain-controlled,
velGrad = -rate I) at 3/s through the gas phase until a contact network carries 1 kPa, then at
config 1's 1/s until the mean stress of Shop::getStress (pkg/dem/Shop_02.cpp:350-376) has
reached 100 kPa at two checks 500 steps apart.  The time step is assemblies.critical_dt's
(0.5 x the smaller of the translational and rotational critical steps).  The oracle runs with
its periodicFix option: the reference applies the torque of a contact across the periodic
boundary to body 2 at its unshifted position and leaves the image's field velocity out of the
relative velocity, which spins particles up without bound (angular velocities of 1e11 rad/s in
this compression); the fixture is a packing with sound dynamics, the workload then runs the
reference's own semantics.  Saved: the
particles' shapes and kinematic state and the cell; the contact history is not saved (the
workload's warm-up steps rebuild the contact angles, and the shear springs restart from zero).

Run: python tests/golden/make_config1_tile.py [threads]
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

N_TILE = 1600
SEED = 11
TARGET_PA = 1e5


def main():
    from oracle import OracleScene
    from sudodem_gb300 import assemblies
    threads = int(sys.argv[1]) if len(sys.argv) > 1 else os.cpu_count()
    # solid fraction at which the lattice spacing (less the +-5% jitter on both sides) exceeds
    # twice the largest bounding radius
    probe = assemblies.periodic_cell(N_TILE, seed=SEED, solid_fraction=0.3, eps_range=(0.3, 1.8))
    rmax = max(assemblies.shape_props(*probe.shape5[p])[4] for p in range(N_TILE))
    m = int(np.ceil(N_TILE ** (1.0 / 3.0)))
    vol = float(np.sum(probe.state[:, 33] / 2650.0))
    spacing = 2.0 * rmax / 0.9 * 1.01
    phi0 = vol / (m * spacing) ** 3
    spec = assemblies.periodic_cell(N_TILE, seed=SEED, solid_fraction=phi0, eps_range=(0.3, 1.8), strain_rate=3.0)
    print(f"start: solid fraction {phi0:.4f}, lattice spacing {spacing * 1e3:.3f} mm", flush=True)
    o = OracleScene.from_spec(spec, threads=threads)
    o.set_periodic_fix(True)
    held = 0
    slow = False
    t0 = time.time()
    chunk = 500
    while True:
        o.step(chunk)
        s = o.get_stress()
        p = -np.trace(s) / 3.0
        L = o.cell()[0]
        print(f"iter {o.iter:7d}  cell {L * 1e3:.4f} mm  phi {vol / L ** 3:.4f}  p {p:.4e} Pa  "
              f"{time.time() - t0:.0f} s", flush=True)
        if not slow and abs(p) >= 1e3:
            o.set_velgrad((-1.0 * np.eye(3)).reshape(9))
            slow = True
        held = held + 1 if abs(p) >= TARGET_PA else 0
        if held >= 2:
            break
    b = o.bodies()
    cell = o.cell()
    np.savez_compressed(os.path.join(HERE, "config1_tile.npz"), shape5=spec.shape5, state=b[:, 0:16],
                        mass_inertia=b[:, 33:37], cell=cell, seed=SEED, iters=o.iter, mean_stress=p, solid_fraction=vol / L ** 3,
                        dt=spec.params["dt"])
    print("saved", os.path.join(HERE, "config1_tile.npz"))


if __name__ == "__main__":
    main()
