"""Builders of the reference's test systems (test/*.jl of NBodySimulator.jl)
and of small synthetic workloads, shared by the oracle and GPU tests."""
import math

import numpy as np

import __graft_entry__ as g

nbg = g.load_package()

KB_KJ = 8.3144598e-3


def lj_two_body():
    """test/lennard_jones_test.jl:4-33"""
    r1 = 1.3
    p1 = nbg.MassBody((-r1 / 2, 0, 0), (0, 0, 0), 1.0)
    p2 = nbg.MassBody((r1 / 2, 0, 0), (0, 0, 0), 1.0)
    params = nbg.LennardJonesParameters(1.0, 1.0, math.inf)
    system = nbg.PotentialNBodySystem([p1, p2], {"lennard_jones": params})
    return nbg.NBodySimulation(system, (0.0, 1.0)), r1


def argon3(bc_kind):
    """test/lennard_jones_test.jl:47-97"""
    T = 120.0
    kb = KB_KJ
    eps = T * kb
    sigma = 0.34
    m = 39.95
    L = 5 * sigma
    R = 2.25 * sigma
    v_dev = math.sqrt(3 * kb * T / m)
    rs = [(L / 3, L / 3, 2 * L / 3), (L / 3, 2 * L / 3, L / 3), (2 * L / 3, L / 3, L / 3)]
    vs = [(0, 0, -v_dev), (0, -v_dev, 0), (-v_dev, 0, 0)]
    bodies = [nbg.MassBody(r, v, m) for r, v in zip(rs, vs)]
    system = nbg.PotentialNBodySystem(bodies, {"lennard_jones": nbg.LennardJonesParameters(eps, sigma, R)})
    bc = nbg.PeriodicBoundaryConditions(L) if bc_kind == "periodic" else nbg.CubicPeriodicBoundaryConditions(L)
    sim = nbg.NBodySimulation(system, (0.0, 100 * 0.5e-3), bc, kb)
    return sim, m, v_dev


def coulomb_pair():
    """test/electrostatics_test.jl:42-68"""
    k = 9.0e9
    q = 1.0e-3
    p1 = nbg.ChargedParticle((-0.5, 0, 0), (0, 0, 0), 1.0, q)
    p2 = nbg.ChargedParticle((0.5, 0, 0), (0, 0, 0), 1.0, q)
    return nbg.NBodySimulation(nbg.ChargedParticles([p1, p2], k), (0.0, 1.0)), k, q


def charges8():
    """test/electrostatics_test.jl:84-119"""
    n = 8
    L = 1.0
    dL = L / (math.ceil(n ** (1 / 3)) + 1)
    grid = []
    x = dL / 2
    while x <= L + 1e-12:
        grid.append(x)
        x += dL
    bodies = []
    for a in grid:
        for b in grid:
            for c in grid:
                if len(bodies) < n:
                    bodies.append(nbg.ChargedParticle((a, b, c), (0, 0, 0), 1.0, 1.0))
    k = 9.0e9
    tau = 0.01 * dL / math.sqrt(2 * k * 1.0 * 1.0 / (dL * 1.0))
    system = nbg.PotentialNBodySystem(bodies, {"electrostatic": nbg.ElectrostaticParameters(k, 0.45 * L)})
    sim = nbg.NBodySimulation(system, (0.0, 1000 * tau), nbg.CubicPeriodicBoundaryConditions(L))
    return sim, tau


def figure8():
    """test/gravitational_test.jl:8-70"""
    m1 = nbg.MassBody((-0.995492, 0, 0), (-0.347902, -0.53393, 0), 1.0)
    m2 = nbg.MassBody((0.995492, 0, 0), (-0.347902, -0.53393, 0), 1.0)
    m3 = nbg.MassBody((0, 0, 0), (0.695804, 1.06786, 0), 1.0)
    return nbg.NBodySimulation(nbg.GravitationalSystem([m1, m2, m3], 1.0), (0.0, 2 * math.pi))


WATER = dict(T=298.16, eps=0.1554253 * 4.184, sigma=0.3165492, rho=997 / 1.6747, mO=15.999, mH=1.00794,
             R=0.9, k_bond=1059.162 * 4.184 * 1.0e2, k_angle=75.9 * 4.184, rOH=0.1012,
             aHOH=113.24 * math.pi / 180, qH=0.41, qO=-0.84, k_el=138.935458, tau=0.5e-3)


def water_params(N=216, Rel_frac=0.49):
    """test/water_test.jl:5-31"""
    w = WATER
    mH2O = w["mO"] + 2 * w["mH"]
    L = (mH2O * N / w["rho"]) ** (1 / 3)
    lj = nbg.LennardJonesParameters(w["eps"], w["sigma"], w["R"])
    el = nbg.ElectrostaticParameters(w["k_el"], Rel_frac * L)
    spc = nbg.SPCFwParameters(w["rOH"], w["aHOH"], w["k_bond"], w["k_angle"])
    return L, lj, el, spc, mH2O


def water3():
    """test/water_test.jl:33-93"""
    w = WATER
    L, lj, el, spc, mH2O = water_params()
    v_dev = math.sqrt(KB_KJ * w["T"] / mH2O)
    rs = [(L / 3, L / 3, 2 * L / 3), (L / 3, 2 * L / 3, L / 3), (2 * L / 3, L / 3, L / 3)]
    vs = [(0, 0, -v_dev), (0, -v_dev, 0), (-v_dev, 0, 0)]
    bodies = [nbg.MassBody(r, v, mH2O) for r, v in zip(rs, vs)]
    water = nbg.WaterSPCFw(bodies, w["mH"], w["mO"], w["qH"], w["qO"], lj, el, spc)
    sim = nbg.NBodySimulation(water, (0.0, 10 * w["tau"]), nbg.CubicPeriodicBoundaryConditions(L), KB_KJ)
    return sim, v_dev, mH2O


def argon125(thermostat, bc_kind="cubic"):
    """test/thermostat_test.jl:1-35 (bodies from this project's seeded generator)"""
    T = 120.0
    kb = KB_KJ
    eps = T * kb
    sigma = 0.34
    rho = 1374 / 1.6747
    m = 39.95
    N = 125
    L = (m * N / rho) ** (1 / 3)
    R = 0.5 * L
    v_dev = math.sqrt(kb * T / m)
    bodies = nbg.generate_bodies_in_cell_nodes(N, m, v_dev, L)
    system = nbg.PotentialNBodySystem(bodies, {"lennard_jones": nbg.LennardJonesParameters(eps, sigma, R)})
    bc = nbg.PeriodicBoundaryConditions(L) if bc_kind == "periodic" else nbg.CubicPeriodicBoundaryConditions(L)
    tau = 0.5e-3
    return nbg.NBodySimulation(system, (0.0, 200 * tau), bc, thermostat, kb, seed=7), tau


def lj_liquid(n=1000, seed=1, rho=0.8, T=1.0, jitter=0.0, skin=0.3, R=2.5, thermostat=None, flags=0):
    pos, vel, L = nbg.workloads.lj_argon_lattice(n, rho=rho, T=T, seed=seed, jitter=jitter)
    bodies = [nbg.MassBody(pos[i], vel[i], 1.0) for i in range(n)]
    system = nbg.PotentialNBodySystem(bodies, {"lennard_jones": nbg.LennardJonesParameters(1.0, 1.0, R)})
    args = [nbg.CubicPeriodicBoundaryConditions(L)]
    if thermostat is not None:
        args.append(thermostat)
    return nbg.NBodySimulation(system, (0.0, 1.0), *args, kb=1.0, skin=skin, flags=flags)


def plummer(n, seed=3, flags=0, mass_spread=0.0):
    """Seeded Plummer sphere; mass_spread > 0 scales each mass by a seeded
    factor in [1 - spread, 1 + spread] (unequal masses)."""
    pos, vel, m = nbg.workloads.plummer_sphere(n, seed=seed)
    if mass_spread:
        m = m * np.random.default_rng(seed + 1).uniform(1.0 - mass_spread, 1.0 + mass_spread, n)
    bodies = [nbg.MassBody(pos[i], vel[i], m[i]) for i in range(n)]
    return nbg.NBodySimulation(nbg.GravitationalSystem(bodies, 1.0), (0.0, 1.0), flags=flags)


def water_box(n_mol, seed=0, eps_rf=1.0, thermostat=None, R=0.9, skin=0.1):
    pos, vel, L = nbg.workloads.spcfw_water_box(n_mol, seed=seed, T=300.0)
    bodies = nbg.workloads.water_molecules(pos, vel)
    lj = nbg.LennardJonesParameters(0.650299, 0.3165492, R)
    el = nbg.ElectrostaticParameters(nbg.workloads.K_EL, R, eps_rf=eps_rf)
    spc = nbg.SPCFwParameters(0.1012, 113.24 * math.pi / 180, nbg.workloads.SPCFW_KB, nbg.workloads.SPCFW_KA)
    water = nbg.WaterSPCFw(bodies, nbg.workloads.M_H, nbg.workloads.M_O, 0.41, -0.82, lj, el, spc)
    args = [nbg.CubicPeriodicBoundaryConditions(L)]
    if thermostat is not None:
        args.append(thermostat)
    return nbg.NBodySimulation(water, (0.0, 1.0), *args, kb=KB_KJ, skin=skin)


def state(sim):
    u0, v0, _ = nbg.gather_bodies_initial_coordinates(sim)
    return u0, v0


def rel_rmse(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def spcfw_water_rf(n_mol, thermo=True, eps_rf=78.5, seed=0, T=300.0):
    """SPC/Fw water (the benchmark parameters) with reaction-field
    electrostatics at 0.9 nm (dielectric eps_rf), Berendsen 300 K or no
    thermostat; the system the learned short-range model is trained on."""
    pos, vel, L = nbg.workloads.spcfw_water_box(n_mol, seed=seed, T=T)
    bodies = nbg.workloads.water_molecules(pos, vel)
    lj = nbg.LennardJonesParameters(0.650299, 0.3165492, 0.9)
    el = nbg.ElectrostaticParameters(nbg.workloads.K_EL, 0.9, eps_rf)
    spc = nbg.SPCFwParameters(0.1012, 113.24 * math.pi / 180, nbg.workloads.SPCFW_KB, nbg.workloads.SPCFW_KA)
    water = nbg.WaterSPCFw(bodies, nbg.workloads.M_H, nbg.workloads.M_O, 0.41, -0.82, lj, el, spc)
    th = nbg.BerendsenThermostat(T, 0.1) if thermo else nbg.NullThermostat()
    sim = nbg.NBodySimulation(water, (0.0, 1.0), nbg.CubicPeriodicBoundaryConditions(L), th,
                              kb=nbg.workloads.KB_KJ, skin=0.1, rebuild_every=10)
    return sim, pos, vel, L
