"""The reference's own physics tests (NBodySimulator.jl test/*.jl), run
through this package's mirror of its API on the GPU engine."""
import math

import numpy as np
import pytest

import systems as S

nbg = S.nbg
pytestmark = pytest.mark.gpu


def test_lj_two_body(gpu):
    sim, r1 = S.lj_two_body()
    res = nbg.run_simulation(sim, nbg.VelocityVerlet(), dt=1e-3)
    r2 = nbg.get_position(res, 1.0, 2) - nbg.get_position(res, 1.0, 1)
    r2n = np.linalg.norm(r2)
    v_expected = math.sqrt(4 * ((1 / r1) ** 12 - (1 / r2n) ** 12 - ((1 / r1) ** 6 - (1 / r2n) ** 6)))
    assert abs(np.linalg.norm(nbg.get_velocity(res, 1.0, 2)) - v_expected) <= 0.001 * v_expected
    assert res.show().endswith("Time steps: 1000\nt: 0.0, 1.0\n")


@pytest.mark.parametrize("bc", ["periodic", "cubic"])
def test_argon3(gpu, bc):
    sim, m, v_dev = S.argon3(bc)
    res = nbg.run_simulation(sim, nbg.VelocityVerlet(), dt=0.5e-3)
    assert abs(nbg.temperature(res, 0.0) - 120.0) < 1e-6
    assert nbg.kinetic_energy(res, 0.0) == pytest.approx(m * 3 * v_dev ** 2 / 2, rel=1e-14)
    e1 = nbg.total_energy(res, 0.0)
    assert abs(nbg.total_energy(res, 100 * 0.5e-3) - e1) <= abs(0.1 * e1)
    assert len(res.solution.t) == 101


def test_coulomb_pair(gpu):
    sim, k, q = S.coulomb_pair()
    res = nbg.run_simulation(sim, nbg.VelocityVerlet(), dt=1e-3)
    r2 = np.linalg.norm(nbg.get_position(res, 1.0, 2) - nbg.get_position(res, 1.0, 1))
    v_expected = math.sqrt(k * q * q * (1 - 1 / r2))
    assert abs(np.linalg.norm(nbg.get_velocity(res, 1.0, 2)) - v_expected) <= 0.001 * v_expected


def test_charges8_energy(gpu):
    sim, tau = S.charges8()
    res = nbg.run_simulation(sim, nbg.VelocityVerlet(), dt=tau, save_everystep=False)
    e1, e2 = nbg.total_energy(res, 0.0), nbg.total_energy(res, sim.tspan[1])
    assert abs((e2 - e1) / e1) <= 1e-3


def test_figure8(gpu):
    sim = S.figure8()
    res = nbg.run_simulation(sim, nbg.VelocityVerlet(), dt=math.pi / 130)
    u = res.solution.u
    assert np.abs(u[-1] - u[0]).max() <= 1e-3
    assert nbg.kinetic_energy(res, 0.0) == pytest.approx(1.218, abs=1e-3)
    r1 = nbg.get_position(res, 0.0, 1)
    assert tuple(r1) == (-0.995492, 0.0, 0.0)
    assert tuple(nbg.get_velocity(res, 0.0, 1)) == (-0.347902, -0.53393, 0.0)


def test_water3(gpu):
    sim, v_dev, mH2O = S.water3()
    w = S.WATER
    t2 = 10 * w["tau"]
    res = nbg.run_simulation(sim, nbg.VelocityVerlet(), dt=w["tau"])
    cc = nbg.get_position(res, t2)
    for i in range(3):
        o = 3 * i
        for h in (1, 2):
            assert abs(w["rOH"] - np.linalg.norm(cc[:, o] - cc[:, o + h])) / w["rOH"] <= 0.01
    e1 = nbg.total_energy(res, 0.0)
    assert e1 == nbg.initial_energy(sim)
    assert abs((e1 - nbg.total_energy(res, t2)) / e1) <= 0.01
    t_expected = 3 * v_dev ** 2 * mH2O / (S.KB_KJ * 21)
    assert abs(nbg.temperature(res, 0.0) - t_expected) / t_expected <= 0.01
    count = 0
    for (r, t) in res:
        assert t == res.solution.t[count]
        count += 1
    assert count == len(res.solution.t)
    ts, d2 = nbg.msd(res)
    assert d2[0] < d2[-1]


@pytest.mark.parametrize("kind", ["andersen", "berendsen", "nosehoover", "langevin"])
def test_thermostats(gpu, kind):
    T0 = 90.0
    tau = 0.5e-3
    if kind == "andersen":
        th, bc, tol, scale, alg = nbg.AndersenThermostat(T0, 0.1 / tau), "periodic", 0.5, T0, nbg.VelocityVerlet()
    elif kind == "berendsen":
        th, bc, tol, scale, alg = nbg.BerendsenThermostat(T0, 10 * tau), "cubic", 0.1, 120.0, nbg.VelocityVerlet()
    elif kind == "nosehoover":
        th, bc, tol, scale, alg = nbg.NoseHooverThermostat(T0, 20 * tau), "cubic", 0.5, T0, nbg.VelocityVerlet()
    else:
        th, bc, tol, scale, alg = nbg.LangevinThermostat(T0, 10.0), "cubic", 0.5, T0, nbg.EM()
    sim, tau = S.argon125(th, bc)
    res = nbg.run_simulation(sim, alg, dt=tau)
    T2 = nbg.temperature(res, 200 * tau)
    assert abs(T2 - T0) / scale <= tol


def test_rdf_peak_and_msd(gpu):
    """lennard_jones_test.jl:120-150: N=125 argon, R = L/2, 400 steps."""
    T = 120.0
    kb = S.KB_KJ
    sigma, m = 0.34, 39.95
    L = 5 * sigma
    bodies = nbg.generate_bodies_in_cell_nodes(125, m, math.sqrt(kb * T / m), L)
    system = nbg.PotentialNBodySystem(bodies, {"lennard_jones": nbg.LennardJonesParameters(T * kb, sigma, 0.5 * L)})
    sim = nbg.NBodySimulation(system, (0.0, 400 * 0.5e-3), nbg.CubicPeriodicBoundaryConditions(L), kb)
    res = nbg.run_simulation(sim, nbg.VelocityVerlet(), dt=0.5e-3, save_every=20)
    ts, d2 = nbg.msd(res)
    assert d2[0] < d2[-1]
    rs, gr = nbg.rdf(res)
    assert abs(rs[int(np.argmax(gr))] / sigma - 1.0) <= 1.0


def test_default_run_simulation_is_adaptive(gpu):
    """gravitational_test.jl:8-24 and electrostatics_test.jl:7-29 call
    run_simulation(simulation) with the default adaptive method: the
    figure-eight back at its start after 2 pi within 0.1, a charge orbit after
    one period within 0.1 r (host DOP853 over the GPU right-hand side)."""
    sim = S.figure8()
    res = nbg.run_simulation(sim)
    u = res.solution.u
    assert res.solution.t[-1] == pytest.approx(2 * math.pi)
    assert np.abs(u[-1] - u[0]).max() <= 0.1
    k, r, q1, q2, m1, m2 = 9.0e9, 100.0, 1.0e-3, -1.0e-3, 100.0, 0.1
    v2 = math.sqrt(abs(k * q1 * q2 / m2 / r))
    p1 = nbg.ChargedParticle((0.0, 0.0, 0.0), (0.0, 0.0, 0.0), m1, q1)
    p2 = nbg.ChargedParticle((r, 0.0, 0.0), (0.0, v2, 0.0), m2, q2)
    sim = nbg.NBodySimulation(nbg.ChargedParticles([p1, p2], k), (0.0, 2 * math.pi * r / v2))
    res = nbg.run_simulation(sim)
    u = res.solution.u
    assert np.abs(u[-1] - u[0]).max() <= 0.1 * r


def test_adaptive_berendsen_matches_oracle_rhs(gpu, oracle):
    """The default adaptive call with a Berendsen thermostat (its right-hand
    side reads v, thermostats.jl:76-83): DOP853 over the GPU right-hand side
    against the same DOP853 driver over the FP64 oracle's right-hand side.
    The two step sequences see forces that differ by FP32 rounding only, so
    the end states agree far inside the integrator's own tolerance."""
    simmod = nbg.simulation
    sim = S.lj_liquid(512, seed=9, jitter=0.05, thermostat=nbg.BerendsenThermostat(1.5, 0.1))
    sim.tspan = (0.0, 0.05)
    res = nbg.run_simulation(sim)
    desc, keep = nbg.system_descriptor(sim)
    u0, v0 = S.state(sim)
    t, tu, tv, nacc = simmod._adaptive_run(lambda v, u, t: oracle.accel(desc, v, u)[0], u0, v0, sim.tspan,
                                           1e-6, 1e-3, False)
    L = desc.box[0]
    assert res.solution.t[-1] == pytest.approx(0.05)
    assert np.abs(np.asarray(res.solution.u[-1]) - tu[-1]).max() <= 1e-6 * L
    assert np.abs(np.asarray(res.solution.v[-1]) - tv[-1]).max() <= 1e-5 * np.abs(tv[-1]).max()
