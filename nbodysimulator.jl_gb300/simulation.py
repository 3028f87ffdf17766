"""NBodySimulation, the ODE/SDE problems, run_simulation and SimulationResult
(mirrors of src/nbody_simulation.jl, src/nbody_to_ode.jl and
src/nbody_simulation_result.jl), with every force, integration and energy
evaluation done by libnbg on the GPU."""
import math
import numbers

import numpy as np

from . import _abi
from .bodies import MassBody, WaterMolecule, is_wide
from .engine import Engine
from .parameters import (AndersenThermostat, BerendsenThermostat,
                         CubicPeriodicBoundaryConditions, InfiniteBox,
                         LangevinThermostat, LennardJonesParameters,
                         NoseHooverThermostat, NullThermostat,
                         PeriodicBoundaryConditions, Thermostat, _jl)
from .systems import (ChargedParticles, GravitationalSystem,
                      PotentialNBodySystem, WaterSPCFw)

kb_SI = 1.38e-23  # nbody_simulation.jl:7


class VelocityVerlet:
    """Velocity Verlet (OrdinaryDiffEqSymplecticRK.VelocityVerlet): fused on
    the GPU by nbg_run."""


class EM:
    """Euler-Maruyama (StochasticDiffEq.EM), used with LangevinThermostat."""


class DOP853:
    """Adaptive Dormand-Prince 8(5,3) (scipy's DOP853) on the host over the
    GPU right-hand side nbg_accel, at SciML's default tolerances (abstol 1e-6,
    reltol 1e-3): what run_simulation(sim) without dt runs. At these
    tolerances scipy's RK45 misses the reference's own closure tests (a charge
    orbit back within 0.1 r); DOP853 meets them. Only the right-hand side runs
    on the GPU; the fused loops are VelocityVerlet, EM and BAOAB."""


class Tsit5(DOP853):
    """The reference's default method name (OrdinaryDiffEqTsit5.Tsit5,
    nbody_simulation_result.jl:480), accepted as an alias of DOP853. Tsit5
    itself is not implemented: the saved times and the accepted-step count
    ("Time steps" in show()) are DOP853's, not the reference's Tsit5 step
    sequence; the states at the saved times agree with the reference within
    the tolerances."""


class BAOAB:
    """Langevin dynamics by the BAOAB splitting (Leimkuhler & Matthews 2013):
    an engine integrator with no reference counterpart, stable at
    velocity-Verlet step sizes where Euler-Maruyama diverges."""


class NBodySimulation:
    """NBodySimulation(system, tspan[, boundary_conditions[, thermostat]][, kb])
    (nbody_simulation.jl:42-125). Engine options (keywords): skin and
    rebuild_every of the Verlet list, seed of the Philox streams, device,
    flags (NBG_FLAG_*)."""

    def __init__(self, system, tspan, *args, kb=None, skin=None, rebuild_every=10, seed=0,
                 device=0, flags=0):
        bc = InfiniteBox()
        thermostat = NullThermostat()
        kb_pos = None
        # arbitrary-precision time span or kb (system_descriptor refuses them)
        self.wide = is_wide(tuple(tspan)) or is_wide(kb) or any(is_wide(a) for a in args)
        for a in args:
            if isinstance(a, (InfiniteBox, CubicPeriodicBoundaryConditions, PeriodicBoundaryConditions)):
                bc = a
            elif isinstance(a, Thermostat):
                thermostat = a
            elif isinstance(a, numbers.Real):
                kb_pos = float(a)
            else:
                raise TypeError(f"unexpected argument {a!r}")
        if isinstance(system, (ChargedParticles, GravitationalSystem)):
            system = PotentialNBodySystem.from_system(system)
        self.system = system
        self.tspan = (float(tspan[0]), float(tspan[1]))
        self.boundary_conditions = bc
        self.thermostat = thermostat
        self.kb = kb if kb is not None else (kb_pos if kb_pos is not None else kb_SI)
        self.skin = skin
        self.rebuild_every = rebuild_every
        self.seed = seed
        self.device = device
        self.flags = flags
        self._engine = None
        self._keep = None

    def show(self):
        out = f"Timespan: ({_jl(self.tspan[0])}, {_jl(self.tspan[1])})\n"
        out += f"Boundary conditions: {self.boundary_conditions.show()}\n"
        if isinstance(self.system, PotentialNBodySystem):
            out += self.system.show()
        return out

    # -- marshalling (nbody_to_ode.jl:1-75, 263-433) ----------------------
    def engine(self):
        if self._engine is None:
            desc, keep = system_descriptor(self)
            self._keep = keep
            self._engine = Engine(desc, self.device)
        return self._engine


def get_masses(system):
    """get_masses (nbody_simulation_result.jl:121-139)."""
    if isinstance(system.bodies, _MassView):
        return system.bodies._m
    if isinstance(system, WaterSPCFw):
        n = len(system.bodies)
        ms = np.empty(3 * n)
        ms[0::3] = system.mO
        ms[1::3] = system.mH
        ms[2::3] = system.mH
        return ms
    return np.array([b.m for b in system.bodies], dtype=np.float64)


def get_coordinate_vector_count(system):
    return 3 * len(system.bodies) if isinstance(system, WaterSPCFw) else len(system.bodies)


def get_degrees_of_freedom(system):
    """(n, nc, ndf) of nbody_simulation_result.jl:152-164."""
    if isinstance(system, WaterSPCFw):
        n = 3 * len(system.bodies)
        nc = 2 * len(system.bodies)
    else:
        n, nc = len(system.bodies), 0
    return n, nc, 3 * n - nc


def gather_bodies_initial_coordinates(simulation):
    """(u0, v0, n) of nbody_to_ode.jl:1-75, as (cols, 3) arrays (the 3 x cols
    column-major layout); with Nose-Hoover one extra zero column."""
    system = simulation.system
    nh = isinstance(simulation.thermostat, NoseHooverThermostat)
    if isinstance(system, WaterSPCFw):
        nm = len(system.bodies)
        cols = 3 * nm + (1 if nh else 0)
        u0 = np.zeros((cols, 3))
        v0 = np.zeros((cols, 3))
        p = system.scpfw_parameters
        for i, b in enumerate(system.bodies):
            o = 3 * i
            if isinstance(b, WaterMolecule):
                u0[o], u0[o + 1], u0[o + 2] = b.O.r, b.H1.r, b.H2.r
                v0[o], v0[o + 1], v0[o + 2] = b.O.v, b.H1.v, b.H2.v
            else:
                u0[o] = b.r
                u0[o + 1] = b.r + np.array([p.rOH, 0.0, 0.0])
                u0[o + 2] = b.r + np.array([math.cos(p.aHOH) * p.rOH, 0.0, math.sin(p.aHOH) * p.rOH])
                v0[o] = v0[o + 1] = v0[o + 2] = b.v
        return u0, v0, nm
    n = len(system.bodies)
    cols = n + (1 if nh else 0)
    u0 = np.zeros((cols, 3))
    v0 = np.zeros((cols, 3))
    for i, b in enumerate(system.bodies):
        u0[i] = b.r
        v0[i] = b.v
    return u0, v0, n


def _has_wide_elements(simulation):
    """Any arbitrary-precision element (is_wide) in the simulation's bodies,
    parameters, time span or kb."""
    sysm = simulation.system
    if getattr(simulation, "wide", False) or any(getattr(b, "wide", False) for b in sysm.bodies):
        return True
    params = list(getattr(sysm, "potentials", {}).values())
    params += [getattr(sysm, a) for a in ("lj_parameters", "e_parameters", "scpfw_parameters") if hasattr(sysm, a)]
    scalars = [getattr(sysm, a) for a in ("mH", "mO", "qH", "qO", "G") if hasattr(sysm, a)]
    return any(is_wide(x) for x in scalars) or any(is_wide(x) for p in params for x in vars(p).values())


def system_descriptor(simulation):
    """Build the nbg_system_desc of a simulation (what the reference's
    obtain_data_for_* functions extract). Returns (desc, keepalive).
    Arbitrary-precision elements (the reference's BigFloat) are refused with
    NBG_ERR_UNSUPPORTED: the caller keeps such a problem on the CPU."""
    if _has_wide_elements(simulation):
        raise _abi.EngineError(-6, "arbitrary-precision elements (BigFloat-like) have no GPU kernel")
    sysm = simulation.system
    d = _abi.NbgSystemDesc()
    d.abi_version = _abi.NBG_ABI_VERSION
    keep = []
    masses = np.ascontiguousarray(get_masses(sysm))
    keep.append(masses)
    d.mass = _abi.as_dptr(masses)
    d.n = len(masses)
    d.lj_cutoff = math.inf
    d.el_cutoff = math.inf
    d.el_eps_rf = 1.0
    if isinstance(sysm, WaterSPCFw):
        d.kind = _abi.NBG_SYSTEM_WATER
        nm = len(sysm.bodies)
        q = np.empty(3 * nm)
        q[0::3] = sysm.qO
        q[1::3] = sysm.qH
        q[2::3] = sysm.qH
        keep.append(q)
        d.charge = _abi.as_dptr(q)
        lj, el, sp = sysm.lj_parameters, sysm.e_parameters, sysm.scpfw_parameters
        d.lj_epsilon, d.lj_sigma, d.lj_cutoff = lj.eps, lj.sigma, lj.R
        d.el_k, d.el_cutoff, d.el_eps_rf = el.k, el.R, getattr(el, "eps_rf", 1.0)
        d.water_rOH, d.water_aHOH, d.water_kb, d.water_ka = sp.rOH, sp.aHOH, sp.kb, sp.ka
        d.potentials = _abi.NBG_POT_LJ | _abi.NBG_POT_EL
    elif isinstance(sysm, PotentialNBodySystem):
        d.kind = _abi.NBG_SYSTEM_POTENTIAL
        pots = sysm.potentials
        mask = 0
        for name in pots:
            if name not in PotentialNBodySystem.ORDER:
                raise _abi.EngineError(-6, f"custom potential {name!r} has no GPU kernel")
        if "lennard_jones" in pots:
            p = pots["lennard_jones"]
            mask |= _abi.NBG_POT_LJ
            d.lj_epsilon, d.lj_sigma, d.lj_cutoff = p.eps, p.sigma, p.R
        if "electrostatic" in pots:
            p = pots["electrostatic"]
            mask |= _abi.NBG_POT_EL
            d.el_k, d.el_cutoff, d.el_eps_rf = p.k, p.R, getattr(p, "eps_rf", 1.0)
            q = np.array([b.q for b in sysm.bodies], dtype=np.float64)
            keep.append(q)
            d.charge = _abi.as_dptr(q)
        if "gravitational" in pots:
            mask |= _abi.NBG_POT_GRAV
            d.grav_G = pots["gravitational"].G
        if "magnetostatic" in pots:
            mask |= _abi.NBG_POT_MAG
            d.mag_mu_4pi = pots["magnetostatic"].mu_4pi
            mm = np.ascontiguousarray(np.array([b.mm for b in sysm.bodies], dtype=np.float64))
            keep.append(mm)
            d.dipole = _abi.as_dptr(mm)
        d.potentials = mask
    else:
        raise _abi.EngineError(-6, f"system {type(sysm).__name__} has no GPU kernels")
    bc = simulation.boundary_conditions
    if isinstance(bc, CubicPeriodicBoundaryConditions):
        d.bc = _abi.NBG_BC_CUBIC
        d.box[0] = bc.L
    elif isinstance(bc, PeriodicBoundaryConditions):
        d.bc = _abi.NBG_BC_PERIODIC
        for k in range(6):
            d.box[k] = bc.boundary[k]
    else:
        d.bc = _abi.NBG_BC_INFINITE
    th = simulation.thermostat
    if isinstance(th, BerendsenThermostat):
        d.thermostat, d.thermo_T, d.thermo_param = _abi.NBG_THERMO_BERENDSEN, th.T, th.tau
    elif isinstance(th, NoseHooverThermostat):
        d.thermostat, d.thermo_T, d.thermo_param = _abi.NBG_THERMO_NOSEHOOVER, th.T, th.tau
    elif isinstance(th, AndersenThermostat):
        d.thermostat, d.thermo_T, d.thermo_param = _abi.NBG_THERMO_ANDERSEN, th.T, th.nu
    elif isinstance(th, LangevinThermostat):
        d.thermostat, d.thermo_T, d.thermo_param = _abi.NBG_THERMO_LANGEVIN, th.T, th.gamma
    else:
        d.thermostat = _abi.NBG_THERMO_NULL
    d.kb = simulation.kb
    d.seed = int(simulation.seed)
    cut = max(d.lj_cutoff if (d.potentials & _abi.NBG_POT_LJ) else 0.0,
              d.el_cutoff if (d.potentials & _abi.NBG_POT_EL) else 0.0)
    d.skin = simulation.skin if simulation.skin is not None else (0.1 * cut if math.isfinite(cut) else 0.0)
    d.rebuild_every = int(simulation.rebuild_every)
    d.flags = int(simulation.flags)
    return d, keep


def lennard_jones_descriptor(masses, L, eps=1.0, sigma=1.0, R=2.5, skin=0.3, thermostat=None, kb=1.0,
                             seed=0, rebuild_every=10):
    """nbg_system_desc of a Lennard-Jones PotentialNBodySystem in a cubic box,
    built straight from a mass array (what system_descriptor extracts from
    the bodies), for large replica ensembles. Returns (desc, keepalive)."""
    masses = np.ascontiguousarray(masses, dtype=np.float64)
    sim = NBodySimulation(PotentialNBodySystem([], {"lennard_jones": LennardJonesParameters(eps, sigma, R)}),
                          (0.0, 1.0), CubicPeriodicBoundaryConditions(L),
                          *( [thermostat] if thermostat is not None else []), kb=kb, skin=skin,
                          rebuild_every=rebuild_every, seed=seed)
    sim.system.bodies = _MassView(masses)
    return system_descriptor(sim)


class _MassView(list):
    """Stand-in body list for lennard_jones_descriptor: only masses are read."""

    class _B:
        __slots__ = ("m",)

        def __init__(self, m):
            self.m = m

    def __init__(self, masses):
        super().__init__()
        self._m = masses

    def __len__(self):
        return len(self._m)


class SecondOrderODEProblem:
    """SciMLBase.SecondOrderODEProblem(sim) (nbody_to_ode.jl:460-536): the
    right-hand side f(dv, v, u, p, t) evaluated by nbg_accel on the GPU, the
    initial state and the time span. Arrays are (cols, 3) float64."""

    def __init__(self, simulation):
        self.simulation = simulation
        self.u0, self.v0, self.n = gather_bodies_initial_coordinates(simulation)
        self.tspan = simulation.tspan
        self._engine = simulation.engine()

    def f(self, dv, v, u, p=None, t=0.0):
        dv[...] = self._engine.accel(v, u, t)

    def __call__(self, v, u, t=0.0):
        return self._engine.accel(v, u, t)


class Solution:
    """Saved frames of a run: t (frames,), u and v (frames, cols, 3)."""

    def __init__(self, t, u, v, naccept):
        self.t = np.asarray(t, dtype=np.float64)
        # every path (fused steps or the host adaptive integrator) stores
        # frames as one (frames, cols, 3) array, so that msd / rdf / the
        # interpolation index them alike
        self.u = np.asarray(u, dtype=np.float64)
        self.v = np.asarray(v, dtype=np.float64)
        self.naccept = naccept


class SimulationResult:
    """SimulationResult(solution, simulation) (nbody_simulation_result.jl:5-8)."""

    def __init__(self, solution, simulation):
        self.solution = solution
        self.simulation = simulation

    def show(self):
        return (f"N: {len(self.simulation.system.bodies)}\n" + self.simulation.show()
                + f"Time steps: {self.solution.naccept}\n"
                + f"t: {_jl(float(self.solution.t.min()))}, {_jl(float(self.solution.t.max()))}\n")

    def __iter__(self):
        for t in self.solution.t:
            yield (self, t)

    def _frame(self, time):
        """State at `time`: the saved frame, or a cubic Hermite interpolant of
        positions (with the saved velocities as derivatives) and a linear one
        of velocities between two frames."""
        ts = self.solution.t
        k = int(np.searchsorted(ts, time))
        tol = 1e-12 * max(1.0, abs(time))
        if k < len(ts) and abs(ts[k] - time) <= tol:
            return self.solution.u[k], self.solution.v[k]
        if k > 0 and abs(ts[k - 1] - time) <= tol:
            return self.solution.u[k - 1], self.solution.v[k - 1]
        if k == 0 or k >= len(ts):
            raise ValueError(f"time {time} outside the saved span")
        t0, t1 = ts[k - 1], ts[k]
        h = t1 - t0
        s = (time - t0) / h
        u0, u1 = self.solution.u[k - 1], self.solution.u[k]
        v0, v1 = self.solution.v[k - 1], self.solution.v[k]
        h00 = 2 * s ** 3 - 3 * s ** 2 + 1
        h10 = s ** 3 - 2 * s ** 2 + s
        h01 = -2 * s ** 3 + 3 * s ** 2
        h11 = s ** 3 - s ** 2
        u = h00 * u0 + h10 * h * v0 + h01 * u1 + h11 * h * v1
        v = (1 - s) * v0 + s * v1
        return u, v


def get_position(sr, time, i=0):
    """Positions (3 x n) at `time`, or of particle i (1-based) when i > 0
    (nbody_simulation_result.jl:90-104)."""
    n = get_coordinate_vector_count(sr.simulation.system)
    u, _ = sr._frame(time)
    return u[:n].T if i <= 0 else u[i - 1].copy()


def get_velocity(sr, time, i=0):
    """Velocities (3 x n) at `time`, or of particle i (1-based) when i > 0
    (nbody_simulation_result.jl:49-71)."""
    n = get_coordinate_vector_count(sr.simulation.system)
    _, v = sr._frame(time)
    return v[:n].T if i <= 0 else v[i - 1].copy()


def _energies(sr, time):
    u, v = sr._frame(time)
    return sr.simulation.engine().energy(u, v)


def temperature(sr, time):
    """md_temperature of the state at `time` (nbody_simulation_result.jl:182-188)."""
    return _energies(sr, time)["temperature"]


def kinetic_energy(sr, time):
    """sum m v^2 / 2 at `time` (nbody_simulation_result.jl:209-218)."""
    return _energies(sr, time)["kinetic"]


def potential_energy(sr, time):
    """potential_energy at `time` (nbody_simulation_result.jl:239-291,399-403):
    LJ + electrostatic (+ bonds + angles for water)."""
    return _energies(sr, time)["potential"]


def total_energy(sr, time):
    """kinetic_energy + potential_energy (nbody_simulation_result.jl:421-425)."""
    return _energies(sr, time)["total"]


def gravitational_energy(sr, time):
    """-G sum_{i<j} m_i m_j / r_ij at `time` (this engine's addition)."""
    return _energies(sr, time)["gravity"]


def initial_energy(simulation):
    """Total energy of the initial condition (nbody_simulation_result.jl:442-446)."""
    u0, v0, _ = gather_bodies_initial_coordinates(simulation)
    return simulation.engine().energy(u0, v0)["total"]


def _adaptive_run(rhs, u0, v0, tspan, abstol, reltol, save_everystep):
    """du = v, dv = rhs(v, u, t) by scipy's DOP853 from (u0, v0) over tspan.
    Returns (t, u frames, v frames, accepted steps): every accepted step, or
    the first and last with save_everystep=False (SciML's saving)."""
    from scipy.integrate import solve_ivp

    shape = u0.shape
    n = u0.size

    def fun(t, y):
        u = y[:n].reshape(shape)
        v = y[n:].reshape(shape)
        return np.concatenate([y[n:], np.asarray(rhs(v.copy(), u.copy(), t), dtype=np.float64).ravel()])

    sol = solve_ivp(fun, (float(tspan[0]), float(tspan[1])), np.concatenate([u0.ravel(), v0.ravel()]),
                    method="DOP853", rtol=reltol, atol=abstol)
    if not sol.success:
        raise RuntimeError(f"adaptive integration failed: {sol.message}")
    keep = np.arange(len(sol.t)) if save_everystep else np.array([0, len(sol.t) - 1])
    y = sol.y.T[keep]
    return (sol.t[keep], [r[:n].reshape(shape) for r in y], [r[n:].reshape(shape) for r in y], len(sol.t) - 1)


def run_simulation(simulation, alg=None, dt=None, save_everystep=True, save_every=None, abstol=1e-6, reltol=1e-3):
    """run_simulation(sim, VelocityVerlet(), dt=...) (nbody_simulation_result.jl:
    468-492). With a LangevinThermostat the first-order SDE is advanced with
    Euler-Maruyama (alg EM()), otherwise with velocity Verlet; both run fused
    on the GPU. The state is saved every step (the reference's default) unless
    save_everystep=False (first and last frame) or save_every=k.

    run_simulation(sim) without dt, or with alg DOP853() (or its alias
    Tsit5()), is the reference's default adaptive call: DOP853 on the host
    over the GPU right-hand side, for systems without a thermostat or with
    Berendsen."""
    if isinstance(alg, DOP853) or (alg is None and dt is None):
        if not isinstance(simulation.thermostat, (NullThermostat, BerendsenThermostat)):
            raise _abi.EngineError(-6, f"{type(simulation.thermostat).__name__} is not integrated adaptively "
                                       "here; use VelocityVerlet (or EM for Langevin) with dt")
        prob = SecondOrderODEProblem(simulation)
        t, tu, tv, nacc = _adaptive_run(prob, prob.u0, prob.v0, simulation.tspan, abstol, reltol, save_everystep)
        return SimulationResult(Solution(t, tu, tv, nacc), simulation)
    if dt is None:
        raise ValueError("dt is required: the GPU integrators take fixed steps")
    if isinstance(alg, BAOAB):
        if not isinstance(simulation.thermostat, LangevinThermostat):
            raise ValueError("BAOAB integrates a LangevinThermostat simulation")
        if not simulation.flags & _abi.NBG_FLAG_LANGEVIN_BAOAB:
            simulation.flags |= _abi.NBG_FLAG_LANGEVIN_BAOAB
            simulation._engine = None
    elif isinstance(simulation.thermostat, LangevinThermostat) and simulation.flags & _abi.NBG_FLAG_LANGEVIN_BAOAB:
        simulation.flags &= ~_abi.NBG_FLAG_LANGEVIN_BAOAB
        simulation._engine = None
    if alg is not None and not isinstance(alg, (VelocityVerlet, EM, BAOAB)):
        raise _abi.EngineError(-6, f"{type(alg).__name__} is not fused on the GPU; use "
                                   "SecondOrderODEProblem(sim) with a host integrator")
    t0, t1 = simulation.tspan
    nsteps = int(round((t1 - t0) / dt))
    if abs(nsteps * dt - (t1 - t0)) > 1e-9 * max(1.0, abs(t1 - t0)):
        nsteps = int(math.ceil((t1 - t0) / dt - 1e-9))
    if save_every is None:
        save_every = 1 if save_everystep else 0
    u0, v0, _ = gather_bodies_initial_coordinates(simulation)
    eng = simulation.engine()
    _, _, tu, tv, stats = eng.run(u0, v0, dt, nsteps, save_every)
    if save_every > 0:
        steps = list(range(0, nsteps + 1, save_every))
        if steps[-1] != nsteps:
            steps.append(nsteps)
    else:
        steps = [0, nsteps] if nsteps > 0 else [0]
    t = [min(t0 + s * dt, t1) for s in steps]
    t[-1] = t1
    return SimulationResult(Solution(t, tu, tv, nsteps), simulation)


def msd(sr):
    """Mean squared displacement over the saved frames
    (nbody_simulation_result.jl:730-783); host-side post-processing."""
    sysm = sr.simulation.system
    ts = sr.solution.t
    U = sr.solution.u
    if isinstance(sysm, WaterSPCFw):
        nm = len(sysm.bodies)
        mO, mH = sysm.mO, sysm.mH
        w = np.array([mO, mH, mH]) / (2 * mH + mO)
        com = (U[:, : 3 * nm].reshape(len(ts), nm, 3, 3) * w[None, None, :, None]).sum(axis=2)
        d = com - com[0]
        return ts, (d * d).sum(axis=2).mean(axis=1)
    n = len(sysm.bodies)
    d = U[:, :n] - U[0, :n]
    return ts, (d * d).sum(axis=2).mean(axis=1)


def rdf(sr, maxbin=1000):
    """Radial distribution function under cubic boundaries
    (nbody_simulation_result.jl:664-709): the pair histogram of every saved
    frame on the GPU (nbg_rdf_histogram), then the reference's normalisation
    by the ideal-gas shell counts. Returns (bin centres, g(r))."""
    sysm = sr.simulation.system
    L = sr.simulation.boundary_conditions.L
    idx = np.arange(0, 3 * len(sysm.bodies), 3) if isinstance(sysm, WaterSPCFw) else np.arange(len(sysm.bodies))
    dr = L / maxbin
    frames = np.ascontiguousarray(np.stack([np.asarray(u, dtype=np.float64) for u in sr.solution.u]))
    hist = _abi.rdf_histogram(frames, idx, L, maxbin)
    n = len(idx)
    c = 4 / 3 * math.pi * n / L ** 3
    rl = np.arange(maxbin) * dr
    nideal = c * ((rl + dr) ** 3 - rl ** 3)
    gr = hist / (len(sr.solution.t) * n) / nideal
    return rl + dr / 2, gr
