"""Shape construction of a superellipsoid on the host, in plain Python.

``shape_props`` restates Superquadrics::Initial (pkg/dem/Superquadrics.cpp:47-93): volume and
geometric inertia from Beta functions, whose log-gamma is the Lanczos approximation with the
Numerical Recipes 3rd-edition coefficients of lib/base/Math.hpp:192-212, and the bounding
radius r_max (times sqrt(2) when an exponent is below 1).  Every operation is the one the C
library ``sqdem_shape_props`` performs, in the same order, on IEEE doubles with the platform's
libm (``math.log/exp/pow``), so the two agree bit for bit on one machine.  Scene generation
(``assemblies``) uses this function so that building an input needs no GPU library.
"""
import math

BODY_STRIDE = 37
INTR_STRIDE = 57

_LANCZOS = (57.1562356658629235, -59.5979603554754912, 14.1360979747417471, -0.491913816097620199,
            .339946499848118887e-4, .465236289270485756e-4, -.983744753048795646e-4, .158088703224912494e-3,
            -.210264441724104883e-3, .217439618115212643e-3, -.164318106536763890e-3, .844182239838527433e-4,
            -.261908384015814087e-4, .368991826595316234e-5)


def gammln(xx):
    """ln Gamma(xx), Lanczos approximation (lib/base/Math.hpp:192-207)."""
    x = y = xx
    tmp = x + 5.24218750000000000
    tmp = (x + 0.5) * math.log(tmp) - tmp
    ser = 0.999999999999997092
    for c in _LANCZOS:
        y += 1.0
        ser += c / y
    return tmp + math.log(2.5066282746310005 * ser / x)


def beta(z, w):
    """B(z, w) = exp(lnG(z) + lnG(w) - lnG(z + w)) (lib/base/Math.hpp:208-212)."""
    return math.exp(gammln(z) + gammln(w) - gammln(z + w))


def shape_props(rx, ry, rz, e1, e2):
    """(volume, Ixx, Iyy, Izz, r_max) of a superellipsoid for unit density."""
    if not (rx > 0 and ry > 0 and rz > 0 and e1 > 0 and e2 > 0):
        raise ValueError("half-axes and exponents must be positive")
    r_max = rx if rx > ry else ry
    r_max = r_max if r_max > rz else rz
    if e1 < 1.0 or e2 < 1.0:
        r_max *= math.pow(2.0, 0.5)
    a = rx * ry * rz * e1 * e2
    beta1 = beta(1.5 * e1, 0.5 * e1) * beta(0.5 * e2, 2. * e2 + 1)
    beta2 = beta(0.5 * e1, 0.5 * e1 + 1) * beta(1.5 * e2, e2 + 1)
    vol = 2. * a * beta(e1 * 0.5, e1 * 0.5) * beta(e2 * 0.5 + 1, e2)
    ixx = 0.5 * a * (math.pow(ry, 2.) * beta1 + 4. * math.pow(rz, 2.) * beta2)
    iyy = 0.5 * a * (math.pow(rx, 2.) * beta1 + 4. * math.pow(rz, 2.) * beta2)
    izz = 0.5 * a * (math.pow(rx, 2.) + math.pow(ry, 2.)) * beta1
    return (vol, ixx, iyy, izz, r_max)
