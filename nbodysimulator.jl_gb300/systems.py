"""N-body systems (mirror of src/nbody_system.jl)."""
from .parameters import (ElectrostaticParameters, GravitationalParameters,
                         LennardJonesParameters, MagnetostaticParameters,
                         PotentialParameters)


class NBodySystem:
    pass


class ChargedParticles(NBodySystem):
    """ChargedParticles(bodies, k) (nbody_system.jl:32-35)."""

    def __init__(self, bodies, k):
        self.bodies = list(bodies)
        self.k = k


class GravitationalSystem(NBodySystem):
    """GravitationalSystem(bodies, G) (nbody_system.jl:61-64)."""

    def __init__(self, bodies, G):
        self.bodies = list(bodies)
        self.G = G


class PotentialNBodySystem(NBodySystem):
    """PotentialNBodySystem(bodies, potentials) with potentials a dict
    {symbol: PotentialParameters}, or a list of built-in names (with default
    parameters) as in nbody_system.jl:72-122. Symbols are strings here
    ("lennard_jones", "electrostatic", "gravitational", "magnetostatic");
    a leading ':' is accepted."""

    ORDER = ("lennard_jones", "electrostatic", "magnetostatic", "gravitational")

    def __init__(self, bodies, potentials=None):
        if isinstance(bodies, (ChargedParticles, GravitationalSystem, PotentialNBodySystem)):
            src = PotentialNBodySystem.from_system(bodies)
            self.bodies, self.potentials = src.bodies, src.potentials
            return
        self.bodies = list(bodies)
        if potentials is None:
            potentials = {}
        if isinstance(potentials, dict):
            self.potentials = {k.lstrip(":"): v for k, v in potentials.items()}
        else:
            names = [p.lstrip(":") for p in potentials]
            self.potentials = {}
            if "lennard_jones" in names:
                self.potentials["lennard_jones"] = LennardJonesParameters()
            if "electrostatic" in names:
                self.potentials["electrostatic"] = ElectrostaticParameters()
            if "gravitational" in names:
                self.potentials["gravitational"] = GravitationalParameters()
            if "magnetostatic" in names:
                self.potentials["magnetostatic"] = MagnetostaticParameters()
        for v in self.potentials.values():
            if not isinstance(v, PotentialParameters):
                raise TypeError("potentials must map names to PotentialParameters")

    @staticmethod
    def from_system(system):
        """PotentialNBodySystem(::ChargedParticles / ::GravitationalSystem)
        (nbody_system.jl:136-150)."""
        if isinstance(system, PotentialNBodySystem):
            return system
        if isinstance(system, ChargedParticles):
            return PotentialNBodySystem(system.bodies, {"electrostatic": ElectrostaticParameters(system.k)})
        if isinstance(system, GravitationalSystem):
            return PotentialNBodySystem(system.bodies, {"gravitational": GravitationalParameters(system.G)})
        raise TypeError(type(system))

    def show(self):
        out = "Potentials: \n"
        for name in self.ORDER:
            if name in self.potentials:
                out += self.potentials[name].show()
        return out


class WaterSPCFw(NBodySystem):
    """WaterSPCFw(bodies, mH, mO, qH, qO, lj_parameters, e_parameters,
    scpfw_parameters) (nbody_system.jl:182-191). bodies are oxygen MassBody
    sites (the hydrogens are placed as in nbody_to_ode.jl:37-55) or explicit
    WaterMolecule triples."""

    def __init__(self, bodies, mH, mO, qH, qO, lj_parameters, e_parameters, scpfw_parameters):
        self.bodies = list(bodies)
        self.mH = mH
        self.mO = mO
        self.qH = qH
        self.qO = qO
        self.lj_parameters = lj_parameters
        self.e_parameters = e_parameters
        self.scpfw_parameters = scpfw_parameters
