"""sudodem_gb300 — GB300-native engines for SudoDEM3D's superellipsoid timestep.

The engines keep the reference's plugin names and attributes (InsertionSortCollider,
Bo1_Superquadrics_Aabb, Bo1_Wall_Aabb, InteractionLoop, Ig2_Superquadrics_Superquadrics_SuperquadricsGeom,
Ig2_Wall_Superquadrics_SuperquadricsGeom, Ip2_SuperquadricsMat_SuperquadricsMat_SuperquadricsPhys,
SuperquadricsLaw, NewtonIntegrator, ForceResetter) so that an ``O.engines`` list written for
SudoDEM3D runs unchanged; the timestep itself runs on the GPU through libsqdem_gpu.so.

The GPU binding (``Engine``, ``Batch``, ``SqdemError``, ``shape_props``) is imported on first
use, so that building inputs with ``assemblies`` touches no native library.
"""
from . import assemblies  # noqa: F401

_NATIVE = ("Batch", "Engine", "SqdemError", "shape_props")


def __getattr__(name):
    if name in _NATIVE:
        from . import _native
        return getattr(_native, name)
    raise AttributeError(f"module 'sudodem_gb300' has no attribute {name!r}")
