"""GB300 force-and-integration engine behind NBodySimulator.jl's API.

Python mirror of the reference's public surface (bodies, systems, potential
parameters, boundary conditions, thermostats, NBodySimulation,
run_simulation and the result analysis), with every force evaluation,
integration step and energy reduction executed by libnbg.so (CUDA, sm_103a)
through the C ABI of include/nbg.h. There is no CPU fallback: without the
built library every compute entry point raises.
"""
from . import _abi
from ._abi import EngineError, load_library
from .bodies import (ChargedParticle, MagneticParticle, MassBody,
                     WaterMolecule, generate_bodies_in_cell_nodes)
from .engine import Engine
from .parameters import (AndersenThermostat, BerendsenThermostat,
                         CubicPeriodicBoundaryConditions,
                         ElectrostaticParameters, GravitationalParameters,
                         InfiniteBox, LangevinThermostat,
                         LennardJonesParameters, MagnetostaticParameters,
                         NoseHooverThermostat, NullThermostat,
                         PeriodicBoundaryConditions, PotentialParameters,
                         SPCFwParameters)
from .simulation import (BAOAB, DOP853, EM, NBodySimulation, SecondOrderODEProblem, Tsit5,
                         SimulationResult, VelocityVerlet,
                         gather_bodies_initial_coordinates, get_masses,
                         get_degrees_of_freedom, get_position, get_velocity,
                         gravitational_energy, initial_energy, kinetic_energy,
                         lennard_jones_descriptor,
                         msd, potential_energy, rdf, run_simulation,
                         system_descriptor, temperature, total_energy, kb_SI)
from .systems import (ChargedParticles, GravitationalSystem,
                      PotentialNBodySystem, WaterSPCFw)
from .pdb import (extract_from_pdb, load_water_molecules_from_pdb,
                  save_to_pdb, write_pdb_data)
from . import workloads

__all__ = [n for n in dir() if not n.startswith("_")]
