"""Seeded synthetic superellipsoid assemblies (the inputs of the benchmarks and tests).

Every assembly is a :class:`SceneSpec`: plain numpy arrays in the body order of the
reference (walls first, ids 0..5, so that the contact-physics wall convention ``id1 <= 5``
of Ip2_SuperquadricsMat_SuperquadricsMat_SuperquadricsPhys holds, pkg/dem/Superquadrics.cpp:1100),
materials and engine parameters.  Bodies are built as NewSuperquadrics_rot2 does
(py/_superquadrics_utils.cpp:354-380): mass = density * volume, inertia = density * geometric
inertia, orientation = the given quaternion normalised; walls as utils.wall
(py/utils.py:311-327): fixed, non-aspherical.

No public dataset is involved; all values come from ``numpy.random.default_rng(seed)``.
"""
from dataclasses import dataclass, field
import math

import numpy as np

from .shapes import BODY_STRIDE, shape_props

_shape_props = shape_props


@dataclass
class SceneSpec:
    kind: np.ndarray            # (N,) 0 superquadric, 1 wall
    shape5: np.ndarray          # (N,5) rx ry rz eps1 eps2
    wall_axis_sense: np.ndarray  # (N,2)
    mat: np.ndarray             # (N,)
    isSphere: np.ndarray        # (N,)
    state: np.ndarray           # (N,37) see include/sqdem.h
    materials: dict             # Kn Ks frictionAngle betan betas density -> (M,)
    params: dict                # sqdem_params fields
    info: dict = field(default_factory=dict)

    @property
    def n_bodies(self):
        return len(self.kind)

    @property
    def n_particles(self):
        return int(np.sum(self.kind == 0))


def _quat_normalize(q):
    # Eigen's normalize: coefficients (x,y,z,w); squaredNorm = (x²+y²)+(z²+w²); divide by sqrt
    w, x, y, z = q
    n2 = (x * x + y * y) + (z * z + w * w)
    n = math.sqrt(n2)
    return np.array([w / n, x / n, y / n, z / n])


def random_quaternions(rng, n):
    """Uniform random unit quaternions (w,x,y,z) from normalised 4-D Gaussians."""
    q = rng.standard_normal((n, 4))
    return np.array([_quat_normalize(qi) for qi in q])


def _builder():
    return {"kind": [], "shape5": [], "was": [], "mat": [], "sph": [], "state": []}


def _add_wall(b, pos, axis, sense, mat=0):
    st = np.zeros(BODY_STRIDE)
    st[0:3] = pos
    st[3] = 1.0
    st[28:31] = np.nan
    b["kind"].append(1); b["shape5"].append(np.zeros(5)); b["was"].append((axis, sense))
    b["mat"].append(mat); b["sph"].append(0); b["state"].append(st)


def _add_sq(b, rxyz, eps, q, pos, density, mat=0, isSphere=0, props_cache=None):
    props = np.asarray(_shape_props(rxyz[0], rxyz[1], rxyz[2], eps[0], eps[1]))
    st = np.zeros(BODY_STRIDE)
    st[0:3] = pos
    st[3:7] = q
    st[28:31] = np.nan
    st[33] = density * props[0]
    st[34:37] = props[1:4] * density
    b["kind"].append(0); b["shape5"].append(np.array([*rxyz, *eps], dtype=np.float64)); b["was"].append((0, 0))
    b["mat"].append(mat); b["sph"].append(isSphere); b["state"].append(st)


def default_params():
    """Timestep parameters at the defaults of the reference's engines: NewtonIntegrator
    (damping 0.2, no gravity, pkg/dem/NewtonIntegrator.hpp:70-89) and InsertionSortCollider
    (verletDist -0.5, targetInterv 50, minSweepDistFactor 0.1, sortAxis 0,
    pkg/common/InsertionSortCollider.hpp:212-222); dt as Scene's default 1e-8."""
    return {"dt": 1e-8, "gravity": (0.0, 0.0, 0.0), "damping": 0.2, "verletDist": -0.5, "targetInterv": 50,
            "minSweepDistFactor": 0.1, "sortAxis": 0, "isSuperquadrics": 1, "exactAsphericalRot": 1}


def _finish(b, materials, params, info):
    return SceneSpec(
        kind=np.array(b["kind"], dtype=np.int32),
        shape5=np.array(b["shape5"], dtype=np.float64).reshape(-1, 5),
        wall_axis_sense=np.array(b["was"], dtype=np.int32).reshape(-1, 2),
        mat=np.array(b["mat"], dtype=np.int32),
        isSphere=np.array(b["sph"], dtype=np.int32),
        state=np.array(b["state"], dtype=np.float64).reshape(-1, BODY_STRIDE),
        materials={k: np.asarray(v, dtype=np.float64) for k, v in materials.items()},
        params=params, info=info)


def default_material(kn=1e5, ks_over_kn=0.5, friction=0.5, density=2650.0):
    return {"Kn": [kn], "Ks": [kn * ks_over_kn], "frictionAngle": [math.atan(friction)], "betan": [0.0],
            "betas": [0.0], "density": [density]}


def critical_dt(spec, factor=0.5, k=None):
    """dt = factor * min over particles of min(sqrt(m / k), sqrt(I_min / (k r_max^2))), k = the
    largest Kn.  The reference has no superquadric critical-dt routine (GlobalStiffnessTimeStepper
    handles ScGeom only).  The rotational term is the period scale of a particle turning about its
    axis of least inertia against a contact spring at its bounding radius: for elongated or
    pointed superellipsoids (eps near 2, aspect ratios up to 1.5) it is 2-5 times shorter than the
    translational sqrt(m / k), and a step above it lets those particles spin up without bound in
    dense packings (the kinetic energy grows until the packing becomes a hot gas)."""
    part = spec.kind == 0
    m = spec.state[part, 33]
    inertia = np.min(spec.state[part, 34:37], axis=1)
    rmax = np.array([shape_props(*s)[4] for s in spec.shape5[part]])
    kk = float(np.max(spec.materials["Kn"])) if k is None else float(k)
    trans = float(np.min(np.sqrt(m / kk)))
    rot = float(np.min(np.sqrt(inertia / (kk * rmax ** 2))))
    return factor * min(trans, rot)


def walled_lattice(n_particles, seed=0, r_range=(0.8e-3, 1.2e-3), eps_range=(0.5, 1.5), spacing=2.6e-3,
                   jitter=0.1e-3, per_side=7, box=None, log_radius=False, friction=0.5, kn=1e5, damping=0.3,
                   verletDist=0.2e-3, lid_height=None, dt_factor=0.5):
    """Particles on a jittered cubic lattice above the floor of a walled box.

    Six walls are created first: x-, x+, y-, y+, floor (sense +1 into the box) and a lid.
    """
    rng = np.random.default_rng(seed)
    side = box if box is not None else per_side * spacing + 2 * (spacing - 0.0002)
    if box is None:
        side = max(side, 20e-3)
    nx = max(1, int(round((side - spacing) / spacing)))
    nx = min(nx, per_side) if box is None else nx
    layers = int(math.ceil(n_particles / (nx * nx)))
    top = spacing * (layers + 1) + 2e-3
    lid = lid_height if lid_height is not None else max(10 * top, 0.2)
    b = _builder()
    _add_wall(b, [0, 0, 0], 0, +1)
    _add_wall(b, [side, 0, 0], 0, -1)
    _add_wall(b, [0, 0, 0], 1, +1)
    _add_wall(b, [0, side, 0], 1, -1)
    _add_wall(b, [0, 0, 0], 2, +1)
    _add_wall(b, [0, 0, lid], 2, -1)
    x0 = side / 2 - (nx - 1) * spacing / 2
    z0 = 2.0e-3 if not log_radius else r_range[1] * math.sqrt(2) + 0.3e-3
    density = 2650.0
    if log_radius:
        r = np.exp(rng.uniform(math.log(r_range[0]), math.log(r_range[1]), size=(n_particles, 3)))
    else:
        r = rng.uniform(r_range[0], r_range[1], size=(n_particles, 3))
    eps = rng.uniform(eps_range[0], eps_range[1], size=(n_particles, 2))
    q = random_quaternions(rng, n_particles)
    jit = rng.uniform(-jitter, jitter, size=(n_particles, 3))
    for p in range(n_particles):
        layer, rem = divmod(p, nx * nx)
        iy, ix = divmod(rem, nx)
        pos = np.array([x0 + ix * spacing, x0 + iy * spacing, z0 + layer * spacing]) + jit[p]
        _add_sq(b, r[p], eps[p], q[p], pos, density)
    mats = default_material(kn=kn, friction=friction, density=density)
    params = {"dt": 1.0, "gravity": (0.0, 0.0, -9.81), "damping": damping, "verletDist": verletDist,
              "targetInterv": 50, "minSweepDistFactor": 0.1, "sortAxis": 0, "isSuperquadrics": 1,
              "exactAsphericalRot": 1}
    spec = _finish(b, mats, params, {"box": side, "layers": layers, "seed": seed})
    spec.params["dt"] = critical_dt(spec, dt_factor)
    return spec


def config0(seed=0, n=1000):
    """1,000 superellipsoids, half-axes U[0.8,1.2] mm, eps U[0.5,1.5], uniform random
    orientations, jittered cubic lattice (2.6 mm, +-0.1 mm) 7x7 per layer above the floor of
    a 20x20 mm walled box; kn=1e5 N/m, ks/kn=0.5, friction 0.5, density 2650, damping 0.3,
    gravity -9.81, dt = 0.5 critical."""
    return walled_lattice(n, seed=seed, box=20e-3, per_side=7)


def per_body_materials(spec, friction=None):
    """Give every body its own copy of material 0 (so that friction, Kn, Ks can differ per
    particle, as the adjoint's per-particle parameters do); friction: per-body coefficients
    (tan of the friction angle) or None to keep material 0's."""
    nb = spec.n_bodies
    m0 = spec.materials
    spec.materials = {k: np.full(nb, float(v[0])) for k, v in m0.items()}
    if friction is not None:
        spec.materials["frictionAngle"] = np.arctan(np.asarray(friction, dtype=np.float64))
    spec.mat = np.arange(nb, dtype=np.int32)
    return spec


def config3(seed=0, n=5000, spacing=3.45e-3, per_side=25):
    """Differentiation specimen: n superellipsoids generated as in config 0 (half-axes U[0.8,1.2]
    mm, eps U[0.5,1.5], uniform random orientations, jittered lattice, kn=1e5 N/m, ks/kn=0.5,
    density 2650, damping 0.3, dt = 0.5 critical) in a square walled box wider than config 0's:
    25 x 25 particles per layer, 8 layers at 5,000 particles (a 20-layer column in a narrow box
    keeps collapsing for ~45,000 steps and its surface outruns a slowly loaded lid), on a 3.45 mm
    lattice (config 0's 2.6 mm lets two boxy particles, eps < 1 and bounding radius up to 1.7 mm,
    overlap at the start, which launches some at up to 2 m/s, 0.2 m high); one material per body
    (the per-particle friction parameters) with friction coefficients U[0.45, 0.55] around config
    0's 0.5: Ip2 gives a pair the smaller of its two friction angles, and with equal values every
    pair sits at the tie of that min, where the loss has no derivative with respect to one
    particle's friction (the one-sided derivatives differ), so the friction gradient needs
    distinct values.  Walls keep 0.5.  The deposition and the lid placement that precede the
    compression window are run by the caller (bench.py's config3 workload)."""
    spec = walled_lattice(n, seed=seed, box=(per_side + 1) * spacing, spacing=spacing)
    mu = np.full(spec.n_bodies, 0.5)
    part = spec.kind == 0
    mu[part] = np.random.default_rng(seed + 7).uniform(0.45, 0.55, int(np.sum(part)))
    return per_body_materials(spec, friction=mu)


def deposition_box(n, seed=0, eps_range=(0.3, 1.8), r_range=(0.8e-3, 1.2e-3), log_radius=False, spacing=2.6e-3):
    """Large walled deposition scene: a square box sized for ~n^(1/3)^2 particles per layer."""
    per_side = max(7, int(round(n ** (1.0 / 3.0) * 1.6)))
    box = per_side * spacing + 2 * (spacing - 0.0002)
    return walled_lattice(n, seed=seed, box=box, per_side=per_side, eps_range=eps_range, r_range=r_range,
                          log_radius=log_radius, spacing=spacing)


def pair_scene(shapeA, shapeB, posA, posB, qA, qB, kn=1e5, friction=0.5, walls=True):
    """Two superellipsoids (plus six far-away walls so ids match the wall convention)."""
    b = _builder()
    if walls:
        far = 1.0
        _add_wall(b, [-far, 0, 0], 0, +1); _add_wall(b, [far, 0, 0], 0, -1)
        _add_wall(b, [0, -far, 0], 1, +1); _add_wall(b, [0, far, 0], 1, -1)
        _add_wall(b, [0, 0, -far], 2, +1); _add_wall(b, [0, 0, far], 2, -1)
    _add_sq(b, shapeA[:3], shapeA[3:5], _quat_normalize(qA), posA, 2650.0)
    _add_sq(b, shapeB[:3], shapeB[3:5], _quat_normalize(qB), posB, 2650.0)
    params = {"dt": 1e-6, "gravity": (0.0, 0.0, 0.0), "damping": 0.0, "verletDist": 0.0, "targetInterv": 50,
              "minSweepDistFactor": 0.1, "sortAxis": 0, "isSuperquadrics": 1, "exactAsphericalRot": 1}
    return _finish(b, default_material(kn=kn, friction=friction), params, {})


def periodic_cell(n_particles, seed=0, solid_fraction=0.3, r_range=(0.8e-3, 1.2e-3), eps_range=(0.3, 1.8),
                  strain_rate=1.0, damping=0.3, kn=1e5, friction=0.5, verletDist=0.2e-3, dt_factor=0.5):
    """Particles on a jittered cubic lattice filling a periodic cube at the given solid
    fraction (the cell side follows from the summed particle volumes), no gravity, and the
    isotropic strain-controlled compression velGrad = -strain_rate * I.  The returned spec
    carries ``info['hSize']`` and ``info['velGrad']`` (row-major 3x3)."""
    rng = np.random.default_rng(seed)
    r = rng.uniform(r_range[0], r_range[1], size=(n_particles, 3))
    eps = rng.uniform(eps_range[0], eps_range[1], size=(n_particles, 2))
    q = random_quaternions(rng, n_particles)
    vol = np.array([_shape_props(*r[p], *eps[p])[0] for p in range(n_particles)])
    L = (vol.sum() / solid_fraction) ** (1.0 / 3.0)
    m = int(math.ceil(n_particles ** (1.0 / 3.0)))
    spacing = L / m
    jit = rng.uniform(-0.05, 0.05, size=(n_particles, 3)) * spacing
    b = _builder()
    density = 2650.0
    for p in range(n_particles):
        iz, rem = divmod(p, m * m)
        iy, ix = divmod(rem, m)
        pos = (np.array([ix, iy, iz]) + 0.5) * spacing + jit[p]
        _add_sq(b, r[p], eps[p], q[p], pos, density)
    mats = default_material(kn=kn, friction=friction, density=density)
    params = {"dt": 1.0, "gravity": (0.0, 0.0, 0.0), "damping": damping, "verletDist": verletDist,
              "targetInterv": 50, "minSweepDistFactor": 0.1, "sortAxis": 0, "isSuperquadrics": 1,
              "exactAsphericalRot": 1}
    hSize = np.diag([L, L, L]).reshape(9)
    velGrad = (-strain_rate * np.eye(3)).reshape(9)
    spec = _finish(b, mats, params, {"periodic": True, "hSize": hSize, "velGrad": velGrad, "cell_side": L,
                                     "seed": seed})
    spec.params["dt"] = critical_dt(spec, dt_factor)
    return spec


def config1(seed=0, n=200_000):
    """200,000 superellipsoids, half-axes U[0.8,1.2] mm, eps1/eps2 U[0.3,1.8], periodic cell at
    initial solid fraction 0.3, isotropic strain-controlled compression (velGrad = -1.0/s * I)."""
    return periodic_cell(n, seed=seed)


def config1_dense(tile_path, tiles=5, strain_rate=1.0):
    """The dense end of config 1: a periodic cell of ``tiles``^3 copies (5: 200,000 particles) of a
    1,600-particle periodic cell of config 1's particles (half-axes U[0.8,1.2] mm, eps U[0.3,1.8])
    compressed isotropically to 100 kPa mean stress (the fixture tests/golden/config1_tile.npz,
    made by tests/golden/make_config1_tile.py), under config 1's loading velGrad =
    -strain_rate I.  Each copy keeps the tile's positions, orientations and velocities (plus the
    affine field velGrad * shift of its place in the larger cell, as a periodic image moves); the
    contact history is not kept (the first steps rebuild the contact angles, the shear springs
    restart from zero)."""
    t = np.load(tile_path)
    shape5, st16, cell = t["shape5"], t["state"], t["cell"]
    h = np.array(cell[0:9]).reshape(3, 3)
    if np.count_nonzero(h - np.diag(np.diag(h))):
        raise ValueError("the tile's cell must be orthogonal")
    Lt = np.diag(h)
    velGrad = -strain_rate * np.eye(3)
    b = _builder()
    density = 2650.0
    n = len(shape5)
    for iz in range(tiles):
        for iy in range(tiles):
            for ix in range(tiles):
                shift = np.array([ix, iy, iz]) * Lt
                for p in range(n):
                    _add_sq(b, shape5[p, 0:3], shape5[p, 3:5], st16[p, 3:7], st16[p, 0:3] + shift, density)
                    row = b["state"][-1]
                    row[7:10] = st16[p, 7:10] + velGrad @ shift
                    row[10:16] = st16[p, 10:16]
    mats = default_material(kn=1e5, friction=0.5, density=density)
    params = {"dt": 1.0, "gravity": (0.0, 0.0, 0.0), "damping": 0.3, "verletDist": 0.2e-3, "targetInterv": 50,
              "minSweepDistFactor": 0.1, "sortAxis": 0, "isSuperquadrics": 1, "exactAsphericalRot": 1}
    hSize = np.diag(Lt * tiles).reshape(9)
    spec = _finish(b, mats, params, {"periodic": True, "hSize": hSize, "velGrad": velGrad.reshape(9),
                                     "cell_side": float(Lt[0] * tiles), "tiles": tiles,
                                     "tile_mean_stress": float(t["mean_stress"]),
                                     "tile_solid_fraction": float(t["solid_fraction"])})
    spec.params["dt"] = critical_dt(spec, 0.5)
    return spec


def cubic_specimen(n_particles, seed=0, friction=0.5, eps_range=(0.4, 1.6), r_range=(0.8e-3, 1.2e-3),
                   spacing=2.6e-3, jitter=0.1e-3, kn=1e5, damping=0.3, verletDist=0.2e-3, dt_factor=0.5,
                   wall_gap=0.2e-3):
    """A closed cubic box of six walls around particles on a jittered cubic lattice, no gravity
    (the specimen of a CompressionEngine test, examples/SudoDEM3D/example2_consol.py:63-93).

    Walls are bodies 0-5 in CompressionEngine's order: left (x-), right (x+), front (y-),
    back (y+), bottom (z-), top (z+), each wall_gap outside the outermost lattice bounds.
    """
    rng = np.random.default_rng(seed)
    nx = max(1, int(math.ceil(n_particles ** (1.0 / 3.0))))
    ny = nx
    nz = int(math.ceil(n_particles / (nx * ny)))
    rmax = r_range[1] * (math.sqrt(2.0) if eps_range[0] < 1.0 else 1.0)
    lo = rmax + wall_gap
    side = [2 * lo + (nx - 1) * spacing, 2 * lo + (ny - 1) * spacing, 2 * lo + (nz - 1) * spacing]
    b = _builder()
    _add_wall(b, [0, 0, 0], 0, +1)
    _add_wall(b, [side[0], 0, 0], 0, -1)
    _add_wall(b, [0, 0, 0], 1, +1)
    _add_wall(b, [0, side[1], 0], 1, -1)
    _add_wall(b, [0, 0, 0], 2, +1)
    _add_wall(b, [0, 0, side[2]], 2, -1)
    density = 2650.0
    r = rng.uniform(r_range[0], r_range[1], size=(n_particles, 3))
    eps = rng.uniform(eps_range[0], eps_range[1], size=(n_particles, 2))
    q = random_quaternions(rng, n_particles)
    jit = rng.uniform(-jitter, jitter, size=(n_particles, 3))
    for p in range(n_particles):
        layer, rem = divmod(p, nx * ny)
        iy, ix = divmod(rem, nx)
        pos = np.array([lo + ix * spacing, lo + iy * spacing, lo + layer * spacing]) + jit[p]
        _add_sq(b, r[p], eps[p], q[p], pos, density)
    mats = default_material(kn=kn, friction=friction, density=density)
    params = {"dt": 1.0, "gravity": (0.0, 0.0, 0.0), "damping": damping, "verletDist": verletDist,
              "targetInterv": 50, "minSweepDistFactor": 0.1, "sortAxis": 0, "isSuperquadrics": 1,
              "exactAsphericalRot": 1}
    spec = _finish(b, mats, params, {"box": side, "seed": seed, "friction": friction})
    spec.params["dt"] = critical_dt(spec, dt_factor)
    return spec


def config2(seed=0, n_specimens=512, n_range=(300, 8000), friction_range=(0.2, 0.8), eps_range=(0.4, 1.6)):
    """512 walled specimens with particle counts log-uniform in [300, 8000] (~1.3M particles),
    friction U[0.2, 0.8] per specimen, eps U[0.4, 1.6]; each a cubic_specimen.  Returns the
    list of specs and the CompressionEngine configuration they run with (100 kPa on the
    lateral walls, axial strain at the top and bottom walls: the shear phase of
    action_cubic, Compression.cpp:485-590).  Particles sit on a 2.1 mm lattice with the walls
    against the outer ones, so most neighbours start in contact."""
    from .servo import servo_config
    rng = np.random.default_rng(seed)
    ns = np.exp(rng.uniform(math.log(n_range[0]), math.log(n_range[1]), size=n_specimens)).astype(int)
    mus = rng.uniform(friction_range[0], friction_range[1], size=n_specimens)
    # dense lattice (2.1 mm) with the walls against the outer particles: a compressed
    # specimen whose contact network is in place from the first step
    specs = [cubic_specimen(int(n), seed=seed * 100003 + i, friction=float(mu), eps_range=eps_range,
                            spacing=2.1e-3, wall_gap=0.0)
             for i, (n, mu) in enumerate(zip(ns, mus))]
    servo = servo_config(z_servo=0, shearMode=1, goalx=1e5, goaly=1e5, goalz=0.05, max_vel=1.0,
                         gain_alpha=0.5, ramp_interval=200, ramp_chunks=20, echo_interval=1000,
                         savedata_interval=1000, target_strain=10.0)
    return specs, servo


def config4(seed=0, n=1_000_000, r_range=(0.5e-3, 2.0e-3), eps_range=(0.2, 1.0), box=0.2, friction=0.5,
            kn=1e5, damping=0.3, verletDist=0.2e-3, dt_factor=0.5):
    """1,000,000 superellipsoids, half-axes log-uniform in [0.5, 2.0] mm, eps U[0.2, 1.0], in a
    200 x 200 mm walled box under gravity (the large deposition case).  Particles are sorted by
    bounding radius and placed layer by layer on square lattices whose spacing is 1.25 times
    the largest bounding radius of the layer (the lattice/size ratio of sq200k_dense: most
    neighbours start in contact, a settled column rather than a free fall).  Six walls first:
    x-, x+, y-, y+, floor and a lid far above."""
    rng = np.random.default_rng(seed)
    r = np.exp(rng.uniform(math.log(r_range[0]), math.log(r_range[1]), size=(n, 3)))
    eps = rng.uniform(eps_range[0], eps_range[1], size=(n, 2))
    q = random_quaternions(rng, n)
    rb = r.max(axis=1) * np.where((eps < 1.0).any(axis=1), math.sqrt(2.0), 1.0)
    order = np.argsort(rb, kind="stable")
    pos = np.zeros((n, 3))
    z = 0.0
    k = 0
    while k < n:
        rmax = rb[order[min(n - 1, k + 1)]]
        sp = 1.25 * rmax
        per = max(1, int((box - 2 * rmax) // sp) + 1)
        take = order[k:k + per * per]
        rl = rb[take].max()
        sp = 1.25 * rl
        per = max(1, int((box - 2 * rl) // sp) + 1)
        take = order[k:k + per * per]
        z += 0.5 * sp if k else 1.02 * rl
        idx = np.arange(len(take))
        iy, ix = np.divmod(idx, per)
        x0 = 0.5 * box - 0.5 * (per - 1) * sp
        pos[take, 0] = x0 + ix * sp
        pos[take, 1] = x0 + iy * sp
        pos[take, 2] = z
        z += 0.5 * sp
        k += len(take)
    b = _builder()
    lid = max(2.0 * z, 0.5)
    _add_wall(b, [0, 0, 0], 0, +1)
    _add_wall(b, [box, 0, 0], 0, -1)
    _add_wall(b, [0, 0, 0], 1, +1)
    _add_wall(b, [0, box, 0], 1, -1)
    _add_wall(b, [0, 0, 0], 2, +1)
    _add_wall(b, [0, 0, lid], 2, -1)
    density = 2650.0
    for p in range(n):
        _add_sq(b, r[p], eps[p], q[p], pos[p], density)
    mats = default_material(kn=kn, friction=friction, density=density)
    params = {"dt": 1.0, "gravity": (0.0, 0.0, -9.81), "damping": damping, "verletDist": verletDist,
              "targetInterv": 50, "minSweepDistFactor": 0.1, "sortAxis": 0, "isSuperquadrics": 1,
              "exactAsphericalRot": 1}
    spec = _finish(b, mats, params, {"box": box, "height": z, "seed": seed})
    spec.params["dt"] = critical_dt(spec, dt_factor)
    return spec


def hertz_mindlin(spec, G=2e8, nu=0.3, dt_factor=0.5, overlap=0.05):
    """The scene with the Hertz-Mindlin contact model (SuperquadricsGeom2, SuperquadricsMat2
    {G, nu}, Ip2_SuperquadricsMat2_SuperquadricsMat2_HertzMindlinPhys, SuperquadricsLaw2).
    Walls (ids 0-5) keep the linear Kn, Ks of their material, as Ip2 gives them.  dt is
    dt_factor * sqrt(m_min / k), k the larger of the wall Kn and the Hertz normal stiffness
    8/3 Gab sqrt(depth R) of the smallest particle pair at the given relative overlap (with the
    rotational term of critical_dt)."""
    m = dict(spec.materials)
    nm = len(m["Kn"])
    m["G"] = np.full(nm, float(G))
    m["nu"] = np.full(nm, float(nu))
    info = dict(spec.info)
    info["contact_model"] = "hertz_mindlin"
    out = SceneSpec(kind=spec.kind, shape5=spec.shape5, wall_axis_sense=spec.wall_axis_sense, mat=spec.mat,
                    isSphere=spec.isSphere, state=spec.state, materials=m, params=dict(spec.params), info=info)
    sq = spec.kind == 0
    rmin = float(np.min(spec.shape5[sq, 0:3]))
    gab = 1.0 / (2 * (1 - nu) / G)
    r_eff = 0.5 * rmin
    k_hm = 8.0 / 3.0 * gab * math.sqrt(overlap * rmin * r_eff)
    k = max(k_hm, float(np.max(m["Kn"])))
    out.params["dt"] = critical_dt(spec, dt_factor, k=k)
    return out
