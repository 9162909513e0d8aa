"""CompressionEngine (pkg/dem/Compression.hpp:39-252) configuration and state layouts.

The engine is passed to the library (``sqdem_set_servo``) and to the CPU oracle as one flat
array of ``SQDEM_SERVO_CONFIG`` doubles, and read back (``sqdem_get_servo``) as one array of
``SQDEM_SERVO_STATE`` doubles.  Names and defaults are the reference's attributes
(Compression.hpp:160-215; ``left_wall_activated`` ... ``top_wall_activated``).
"""
import numpy as np

CONFIG_FIELDS = (
    ("enabled", 1.0), ("z_servo", 1.0), ("continueFlag", 0.0), ("hydroStrain", 0.0), ("shearMode", 1.0),
    ("left_wall_activated", 1.0), ("right_wall_activated", 1.0), ("front_wall_activated", 1.0),
    ("back_wall_activated", 1.0), ("bottom_wall_activated", 1.0), ("top_wall_activated", 1.0),
    ("iterate_num_max", 100.0), ("solve_num_max", 2000.0), ("echo_interval", 1000.0), ("savedata_interval", 12.0),
    ("ramp_interval", 10000.0), ("ramp_chunks", 400.0),
    ("goalx", 0.0), ("goaly", 0.0), ("goalz", 0.0),
    ("gain_alpha", 0.5), ("target_strain", 0.15), ("f_threshold", 0.01), ("fmin_threshold", 0.01),
    ("unbf_tol", 0.01), ("max_vel", 1.0), ("hydroStrainRate", 0.0),
    ("width0", 0.0), ("height0", 0.0), ("depth0", 0.0),
)
CONFIG_NAMES = tuple(n for n, _ in CONFIG_FIELDS)
CONFIG_SIZE = len(CONFIG_FIELDS)          # SQDEM_SERVO_CONFIG

STATE_NAMES = (
    "width", "depth", "height", "x_area", "y_area", "z_area", "wsxx", "wsyy", "wszz",
    "wsxx_left", "wsxx_right", "wsyy_front", "wsyy_back", "wszz_bottom", "wszz_top",
    "gain_x", "gain_x1", "gain_y", "gain_y1", "gain_z", "gain_z1", "UnbalancedForce",
    "particlesVolume", "Init_boxVolume", "Current_boxVolume", "strain2",
    "iterate_num", "solve_num", "rampNum", "Flag_ForceTarget", "firstRun", "width0", "height0", "depth0",
    "stopAtIter", "quiet_system_flag",
)
STATE_SIZE = len(STATE_NAMES)             # SQDEM_SERVO_STATE


def servo_config(**kw):
    """Flat configuration array; unknown names raise (as the reference's attribute setter)."""
    out = np.array([v for _, v in CONFIG_FIELDS], dtype=np.float64)
    for k, v in kw.items():
        if k not in CONFIG_NAMES:
            raise AttributeError("CompressionEngine has no attribute %r" % k)
        out[CONFIG_NAMES.index(k)] = float(v)
    return out


def state_dict(arr):
    return {n: float(arr[i]) for i, n in enumerate(STATE_NAMES)}
