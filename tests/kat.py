"""Known-answer narrowphase construction (the PositionPB idea of the reference,
py/_superquadrics_utils.cpp:109-131, applied to superellipsoids).

Pick surface angles on body A; its outward normal n and surface point pA are known in
closed form (Superquadrics.cpp:110-120, 258-266).  Place body B so that its support point
along -n sits at pA - n*delta.  Then the exact answer is: contact normal n, penetration
depth delta, contact point pA - n*delta/2.
"""
import math

import numpy as np

import oracle as O
from sudodem_gb300 import assemblies


def rot(q):
    w, x, y, z = q
    tx, ty, tz = 2 * x, 2 * y, 2 * z
    return np.array([[1 - (ty * y + tz * z), ty * x - tz * w, tz * x + ty * w],
                     [ty * x + tz * w, 1 - (tx * x + tz * z), tz * y - tx * w],
                     [tz * x - ty * w, tz * y + tx * w, 1 - (tx * x + ty * y)]])


def make_case(rng, eps_range=(0.3, 1.8), delta_rel=1e-5, r_range=(0.8e-3, 1.2e-3)):
    sA = np.array([*rng.uniform(*r_range, 3), *rng.uniform(*eps_range, 2)])
    sB = np.array([*rng.uniform(*r_range, 3), *rng.uniform(*eps_range, 2)])
    qA = assemblies.random_quaternions(rng, 1)[0]
    qB = assemblies.random_quaternions(rng, 1)[0]
    RA, RB = rot(qA), rot(qB)
    ph = (rng.uniform(-math.pi, math.pi), rng.uniform(-1.3, 1.3))
    nA = O.normal(sA, *ph)
    nA = nA / np.linalg.norm(nA)
    pA_loc = O.surface(sA, *ph)
    n = RA @ nA
    posA = rng.uniform(-1e-3, 1e-3, 3)
    pA = RA @ pA_loc + posA
    mB = RB.T @ (-n)
    psi = O.normal2phi(sB, mB)
    sBp = O.surface(sB, *psi)
    delta = delta_rel * float(np.max(sA[:3]))
    posB = (pA - n * delta) - RB @ sBp
    return sA, sB, qA, qB, posA, posB, n, delta, pA - n * delta / 2
