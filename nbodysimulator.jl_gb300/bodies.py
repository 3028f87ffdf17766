"""Bodies of an n-body system (mirror of src/bodies.jl).

Positions and velocities are length-3 float64 arrays, as the reference's
SVector{3} fields.
"""
import decimal
import fractions
import math

import numpy as np


def is_wide(x):
    """True for an element type wider than float64, the counterpart of the
    reference's BigFloat (and exact Rational) support: Decimal, Fraction,
    mpmath numbers, numpy longdouble, or a container holding one. Such
    problems have no GPU kernel; float32 and float64 inputs are computed in
    float64."""
    if isinstance(x, (decimal.Decimal, fractions.Fraction)):
        return True
    if type(x).__module__.split(".")[0] == "mpmath":
        return True
    if isinstance(x, np.ndarray):
        if x.dtype == object:
            return any(is_wide(e) for e in x.flat)
        return (x.dtype.kind == "f" and x.dtype.itemsize > 8) or (x.dtype.kind == "c" and x.dtype.itemsize > 16)
    if isinstance(x, np.generic):
        return is_wide(np.asarray(x))
    if isinstance(x, (list, tuple)):
        return any(is_wide(e) for e in x)
    return False


def _vec3(x):
    a = np.asarray(x, dtype=np.float64).reshape(3)
    return a.copy()


class Body:
    pass


class MassBody(Body):
    """MassBody(r, v, m) (bodies.jl:37)."""

    def __init__(self, r, v, m):
        self.wide = is_wide(r) or is_wide(v) or is_wide(m)
        self.r = _vec3(r)
        self.v = _vec3(v)
        self.m = float(m)


class ChargedParticle(Body):
    """ChargedParticle(r, v, m, q) (bodies.jl:68)."""

    def __init__(self, r, v, m, q):
        self.wide = is_wide(r) or is_wide(v) or is_wide(m) or is_wide(q)
        self.r = _vec3(r)
        self.v = _vec3(v)
        self.m = float(m)
        self.q = float(q)


class MagneticParticle(Body):
    """MagneticParticle(r, v, m, mm) with magnetic moment mm (bodies.jl:102-107)."""

    def __init__(self, r, v, m, mm):
        self.wide = is_wide(r) or is_wide(v) or is_wide(m) or is_wide(mm)
        self.r = _vec3(r)
        self.v = _vec3(v)
        self.m = float(m)
        self.mm = _vec3(mm)


class WaterMolecule(Body):
    """WaterMolecule(O, H1, H2) of three MassBody sites (bodies.jl:109-113)."""

    def __init__(self, O, H1, H2):
        self.O = O
        self.H1 = H1
        self.H2 = H2
        self.wide = any(getattr(b, "wide", False) for b in (O, H1, H2))


def generate_bodies_in_cell_nodes(n, m, v_dev, L, rng=None):
    """n equal-mass bodies on a cubic grid with normal velocities
    (bodies.jl:139-159): spacing dL = L / ceil(n^(1/3)), sites at
    dL/2, dL/2 + dL, ... <= L with x outermost and z innermost,
    v = v_dev * randn. Julia's MersenneTwister(n) stream is not reproducible
    here, so the velocities come from numpy's PCG64 seeded with n unless an
    rng is given."""
    if rng is None:
        rng = np.random.default_rng(n)
    velocities = v_dev * rng.standard_normal((n, 3))
    side = math.ceil(n ** (1.0 / 3.0) - 1e-12)
    dL = L / side
    coords = []
    k = 0
    while True:
        c = dL / 2 + k * dL
        if c > L * (1 + 1e-15):
            break
        coords.append(c)
        k += 1
    bodies = []
    count = 0
    for x in coords:
        for y in coords:
            for z in coords:
                if count >= n:
                    return bodies
                bodies.append(MassBody((x, y, z), velocities[count], m))
                count += 1
    return bodies
