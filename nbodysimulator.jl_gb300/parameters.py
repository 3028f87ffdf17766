"""Potential parameters, boundary conditions and thermostats
(mirrors of src/basic_potentials.jl:33-238, src/boundary_conditions.jl and
src/thermostats.jl). The show() strings follow the reference's Base.show."""
import math


def _jl(x):
    """Julia's show of a Real: 1.0, 2, Inf, 9.0e9, 6.67408e-11."""
    if isinstance(x, bool):
        return str(x).lower()
    if isinstance(x, int):
        return str(x)
    if math.isinf(x):
        return "Inf" if x > 0 else "-Inf"
    if math.isnan(x):
        return "NaN"
    x = float(x)
    if x == 0.0:
        return "-0.0" if math.copysign(1.0, x) < 0 else "0.0"
    # shortest round-trip digits, then Julia's layout: scientific notation
    # when the decimal exponent is >= 6 or < -4, else plain with ".0"
    mant, ex = f"{x:.17e}".split("e")
    r = repr(x)
    digits = r.replace("-", "").split("e")[0].replace(".", "").lstrip("0") or "0"
    exp10 = int(ex)
    if "e" in r:
        m, e = r.split("e")
        digits = m.replace("-", "").replace(".", "").lstrip("0")
        exp10 = int(e) + (len(m.replace("-", "").split(".")[0]) - 1)
    digits = digits.rstrip("0") or "0"
    sign = "-" if x < 0 else ""
    if exp10 >= 6 or exp10 < -4:
        m = digits[0] + "." + (digits[1:] or "0")
        return f"{sign}{m}e{exp10}"
    if "e" in r:
        return repr(float(f"{x:.17g}")) if "e" not in repr(float(f"{x:.17g}")) else f"{x:f}"
    return r


class PotentialParameters:
    """Abstract potential-parameter type (basic_potentials.jl:1-33)."""


class LennardJonesParameters(PotentialParameters):
    """LennardJonesParameters(eps=1, sigma=1, R=2.5) caching sigma^2 and R^2
    (basic_potentials.jl:59-73)."""

    def __init__(self, eps=1.0, sigma=1.0, R=2.5):
        self.eps = eps
        self.sigma = sigma
        self.R = R
        self.sigma2 = sigma ** 2
        self.R2 = R ** 2

    def show(self):
        return f"Lennard-Jones:\n\tϵ:{_jl(self.eps)}\n\tσ:{_jl(self.sigma)}\n\tR:{_jl(self.R)}\n"


class GravitationalParameters(PotentialParameters):
    """GravitationalParameters(G=6.67408e-11) (basic_potentials.jl:109-115)."""

    def __init__(self, G=6.67408e-11):
        self.G = G

    def show(self):
        return f"Gravitational:\n\tG:{_jl(self.G)}\n"


class ElectrostaticParameters(PotentialParameters):
    """ElectrostaticParameters(k=9e9, R=Inf) (basic_potentials.jl:147-163).
    eps_rf is this engine's reaction-field dielectric; 1.0 (the default)
    reproduces the reference's truncated Coulomb force exactly."""

    def __init__(self, k=9.0e9, R=math.inf, eps_rf=1.0):
        self.k = k
        self.R = R
        self.R2 = R ** 2
        self.eps_rf = eps_rf

    def show(self):
        return f"Electrostatic:\n\tk:{_jl(self.k)}\n"


class MagnetostaticParameters(PotentialParameters):
    """MagnetostaticParameters(mu_4pi=1e-7) (basic_potentials.jl:193-199)."""

    def __init__(self, mu_4pi=1.0e-7):
        self.mu_4pi = mu_4pi

    def show(self):
        return f"Magnetostatic:\n\tμ/4π:{_jl(self.mu_4pi)}\n"


class SPCFwParameters(PotentialParameters):
    """SPCFwParameters(rOH, aHOH, kb, ka) (basic_potentials.jl:233-238)."""

    def __init__(self, rOH, aHOH, kb, ka):
        self.rOH = rOH
        self.aHOH = aHOH
        self.kb = kb
        self.ka = ka


class BoundaryConditions:
    pass


class InfiniteBox(BoundaryConditions):
    """InfiniteBox (boundary_conditions.jl): plain differences."""

    def __init__(self, boundary=(-math.inf, math.inf) * 3):
        self.boundary = list(boundary)

    def show(self):
        return "InfiniteBox{Float64}([" + ", ".join(_jl(float(b)) for b in self.boundary) + "])"


class CubicPeriodicBoundaryConditions(BoundaryConditions):
    """CubicPeriodicBoundaryConditions(L): minimum image by repeated +-L
    (boundary_conditions.jl:101-165)."""

    def __init__(self, L):
        self.L = L

    def show(self):
        return f"CubicPeriodicBoundaryConditions{{Float64}}({_jl(float(self.L))})"


class PeriodicBoundaryConditions(BoundaryConditions):
    """PeriodicBoundaryConditions(L) or ([lo,hi] x 3): differences mapped into
    [lo, hi) (boundary_conditions.jl:111-136)."""

    def __init__(self, *args):
        if len(args) == 1 and not hasattr(args[0], "__len__"):
            L = float(args[0])
            self.boundary = [0.0, L, 0.0, L, 0.0, L]
        else:
            b = args[0] if len(args) == 1 else args
            self.boundary = [float(x) for x in b]

    def __getitem__(self, i):
        """1-based indexing like the reference's getindex."""
        return self.boundary[i - 1]

    def __iter__(self):
        return iter(self.boundary)

    def show(self):
        return "PeriodicBoundaryConditions{Float64}([" + ", ".join(_jl(b) for b in self.boundary) + "])"


class Thermostat:
    pass


class NullThermostat(Thermostat):
    pass


class AndersenThermostat(Thermostat):
    """AndersenThermostat(T, nu) (thermostats.jl:37-40)."""

    def __init__(self, T, nu):
        self.T = T
        self.nu = nu


class BerendsenThermostat(Thermostat):
    """BerendsenThermostat(T, tau) with gamma = 0.5 / tau (thermostats.jl:66-74)."""

    def __init__(self, T, tau):
        self.T = T
        self.tau = tau
        self.gamma = 0.5 / tau


class NoseHooverThermostat(Thermostat):
    """NoseHooverThermostat(T, tau) (thermostats.jl:116-119)."""

    def __init__(self, T, tau):
        self.T = T
        self.tau = tau


class LangevinThermostat(Thermostat):
    """LangevinThermostat(T, gamma) (thermostats.jl:153-156)."""

    def __init__(self, T, gamma):
        self.T = T
        self.gamma = gamma
