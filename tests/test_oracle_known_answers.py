"""The FP64 oracle against the known answers of the reference's own tests
(NBodySimulator.jl test/*.jl). These pin the oracle before it is used as
the oracle of the GPU engine. CPU only."""
import math

import numpy as np
import pytest

import systems as S

nbg = S.nbg


def _run(oracle, sim, dt, nsteps, save_every=0):
    desc, keep = nbg.system_descriptor(sim)
    u0, v0 = S.state(sim)
    u, v = oracle.run(desc, u0, v0, dt, nsteps, save_every)
    return desc, keep, u0, v0, u, v


def test_lj_two_body_speed(oracle):
    """lennard_jones_test.jl:4-33: speed from energy conservation, 0.1 %."""
    sim, r1 = S.lj_two_body()
    desc, keep, u0, v0, u, v = _run(oracle, sim, 1e-3, 1000)
    r2 = np.linalg.norm(u[1] - u[0])
    v_expected = math.sqrt(4 * 1.0 / 1.0 * ((1 / r1) ** 12 - (1 / r2) ** 12 - ((1 / r1) ** 6 - (1 / r2) ** 6)))
    assert abs(np.linalg.norm(v[1]) - v_expected) <= 0.001 * v_expected


@pytest.mark.parametrize("bc", ["periodic", "cubic"])
def test_argon3_temperature_energy(oracle, bc):
    """lennard_jones_test.jl:47-97: T(0)=120 K, kinetic energy, 10 % energy drift."""
    sim, m, v_dev = S.argon3(bc)
    desc, keep, u0, v0, u, v = _run(oracle, sim, 0.5e-3, 100)
    e0 = oracle.energy(desc, u0, v0)
    assert abs(e0["temperature"] - 120.0) < 1e-6
    assert e0["kinetic"] == pytest.approx(m * 3 * v_dev ** 2 / 2, rel=1e-14)
    e1 = oracle.energy(desc, u, v)
    assert abs(e1["total"] - e0["total"]) <= abs(0.1 * e0["total"])


def test_coulomb_repulsion_speed(oracle):
    """electrostatics_test.jl:42-68: speed from energy conservation, 0.1 %."""
    sim, k, q = S.coulomb_pair()
    desc, keep, u0, v0, u, v = _run(oracle, sim, 1e-3, 1000)
    r2 = np.linalg.norm(u[1] - u[0])
    v_expected = math.sqrt(k * q * q / 1.0 * (1 / 1.0 - 1 / r2))
    assert abs(np.linalg.norm(v[1]) - v_expected) <= 0.001 * v_expected


def test_charges8_energy_conservation(oracle):
    """electrostatics_test.jl:84-119: 8 charges, cubic box, cutoff 0.45 L,
    1000 VV steps, relative drift within 1e-3."""
    sim, tau = S.charges8()
    desc, keep, u0, v0, u, v = _run(oracle, sim, tau, 1000)
    e0 = oracle.energy(desc, u0, v0)["total"]
    e1 = oracle.energy(desc, u, v)["total"]
    assert abs((e1 - e0) / e0) <= 1e-3


def test_figure8_vv_closure(oracle):
    """gravitational_test.jl:53-60 and :218-220: VV dt=pi/130 returns the
    figure-eight to its start within 1e-3; KE(0) = 1.218 within 1e-3."""
    sim = S.figure8()
    desc, keep, u0, v0, u, v = _run(oracle, sim, math.pi / 130, 260)
    assert np.abs(u - u0).max() <= 1e-3
    assert oracle.energy(desc, u0, v0)["kinetic"] == pytest.approx(1.218, abs=1e-3)


def test_water3_geometry_energy_temperature(oracle):
    """water_test.jl:33-93: 3 SPC/Fw molecules, 10 VV steps: bonds and angle
    within 1 %, total energy drift within 1 %, T(0) with ndf = 21."""
    sim, v_dev, mH2O = S.water3()
    w = S.WATER
    desc, keep, u0, v0, u, v = _run(oracle, sim, w["tau"], 10)
    for i in range(3):
        o = 3 * i
        for h in (1, 2):
            assert abs(w["rOH"] - np.linalg.norm(u[o] - u[o + h])) / w["rOH"] <= 0.01
        a, b = u[o] - u[o + 1], u[o] - u[o + 2]
        ang = math.acos(a @ b / (np.linalg.norm(a) * np.linalg.norm(b)))
        assert abs(ang - w["aHOH"]) / w["aHOH"] <= 0.01
    e0 = oracle.energy(desc, u0, v0)
    e1 = oracle.energy(desc, u, v)
    assert abs((e0["total"] - e1["total"]) / e0["total"]) <= 0.01
    t_expected = 3 * v_dev ** 2 * mH2O / (S.KB_KJ * 21)
    assert abs(e0["temperature"] - t_expected) / t_expected <= 0.01


@pytest.mark.parametrize("kind", ["andersen", "berendsen", "nosehoover", "langevin"])
def test_thermostats_argon125(oracle, kind):
    """thermostat_test.jl:16-94: N=125 argon, 200 steps towards T0 = 90 K."""
    T0 = 90.0
    tau = 0.5e-3
    if kind == "andersen":
        th, bc, tol, scale = nbg.AndersenThermostat(T0, 0.1 / tau), "periodic", 0.5, T0
    elif kind == "berendsen":
        th, bc, tol, scale = nbg.BerendsenThermostat(T0, 10 * tau), "cubic", 0.1, 120.0
    elif kind == "nosehoover":
        th, bc, tol, scale = nbg.NoseHooverThermostat(T0, 20 * tau), "cubic", 0.5, T0
    else:
        th, bc, tol, scale = nbg.LangevinThermostat(T0, 10.0), "cubic", 0.5, T0
    sim, tau = S.argon125(th, bc)
    desc, keep, u0, v0, u, v = _run(oracle, sim, tau, 200)
    T2 = oracle.energy(desc, u, v)["temperature"]
    assert abs(T2 - T0) / scale <= tol


def test_baoab_thermostat_argon125(oracle):
    """The BAOAB Langevin option reaches T0 on the thermostat test's argon
    (gamma = 10, as thermostat_test.jl:197-214)."""
    th = nbg.LangevinThermostat(90.0, 10.0)
    sim, tau = S.argon125(th, "cubic")
    sim.flags |= nbg._abi.NBG_FLAG_LANGEVIN_BAOAB
    desc, keep, u0, v0, u, v = _run(oracle, sim, tau, 200)
    T2 = oracle.energy(desc, u, v)["temperature"]
    assert abs(T2 - 90.0) / 90.0 <= 0.5


def test_philox_streams_distinct(oracle):
    """The counter-based RNG gives distinct, well-spread draws."""
    us = np.array([oracle.uniform(7, i, 0) for i in range(2000)])
    assert 0.45 < us.mean() < 0.55
    zs = np.array([oracle.normals3(7, i, 3) for i in range(2000)]).ravel()
    assert abs(zs.mean()) < 0.06 and abs(zs.std() - 1) < 0.05


def _rdf_loops(frames, idx, L, maxbin):
    """The reference rdf's loops (nbody_simulation_result.jl:672-692) with its
    minimum image (boundary_conditions.jl:138-165), in plain Python."""
    hist = [0.0] * maxbin
    dr = L / maxbin
    radius = 0.5 * L
    for cc in frames:
        for a in range(len(idx)):
            ri = cc[idx[a]]
            for b in range(a + 1, len(idx)):
                rj = cc[idx[b]]
                d = [float(ri[k]) - float(rj[k]) for k in range(3)]
                for k in range(3):
                    while d[k] >= radius:
                        d[k] -= L
                    while d[k] < -radius:
                        d[k] += L
                r2 = d[0] ** 2 + d[1] ** 2 + d[2] ** 2
                if r2 < (0.5 * L) ** 2:
                    bn = math.ceil(math.sqrt(r2) / dr)
                    if 1 < bn <= maxbin:
                        hist[bn - 1] += 2
    return np.array(hist)


@pytest.mark.parametrize("maxbin", [1000, 37])
def test_rdf_histogram_oracle_matches_reference_loops(oracle, maxbin):
    """The oracle's rdf histogram equals the reference's loops on unwrapped
    frames, bin-edge distances and a ragged participant subset."""
    rng = np.random.default_rng(maxbin)
    L = 3.0
    frames = rng.uniform(-2 * L, 3 * L, size=(2, 60, 3))
    dr = L / maxbin
    frames[0, 1] = frames[0, 0] + [dr * 7, 0.0, 0.0]       # on a bin edge
    frames[0, 2] = frames[0, 0] + [0.5 * L, 0.0, 0.0]      # half the box
    frames[1, 3] = frames[1, 4] + [0.0, 11 * dr, 0.0]
    idx = np.concatenate([np.arange(0, 60, 2), [1, 3]])
    ref = _rdf_loops(frames, idx, L, maxbin)
    prev = oracle.lib().oracle_get_threads()
    try:
        for nt in (1, 4):
            oracle.set_threads(nt)
            assert np.array_equal(oracle.rdf_histogram(frames, idx, L, maxbin), ref)
    finally:
        oracle.set_threads(prev)


def test_charge_orbit_closure(oracle):
    """electrostatics_test.jl:7-40: a light negative charge on a circular
    orbit around a heavy positive one returns to its start after one period,
    within 0.1 r (the reference integrates with its default adaptive method;
    velocity Verlet at T / 2000 here)."""
    k, r, q1, q2, m1, m2 = 9.0e9, 100.0, 1.0e-3, -1.0e-3, 100.0, 0.1
    v2 = math.sqrt(abs(k * q1 * q2 / m2 / r))
    period = 2 * math.pi * r / v2
    p1 = nbg.ChargedParticle((0.0, 0.0, 0.0), (0.0, 0.0, 0.0), m1, q1)
    p2 = nbg.ChargedParticle((r, 0.0, 0.0), (0.0, v2, 0.0), m2, q2)
    sim = nbg.NBodySimulation(nbg.ChargedParticles([p1, p2], k), (0.0, period))
    desc, keep, u0, v0, u, v = _run(oracle, sim, period / 2000, 2000)
    assert np.abs(u - u0).max() <= 0.1 * r


def test_five_body_choreography_closure(oracle):
    """gravitational_test.jl:72-101: the 5-body choreography returns to its
    start after t = 2 pi within 0.01 (the reference integrates with Tsit5 at
    1e-10 tolerances; velocity Verlet at 2 pi / 200000 here: the six-digit
    initial conditions leave ~0.005 at t = 2 pi for any fine step)."""
    rs = [(1.657666, 0.0, 0.0), (0.439775, -0.169717, 0.0), (-1.268608, -0.267651, 0.0),
          (-1.268608, 0.267651, 0.0), (0.439775, 0.169717, 0.0)]
    vs = [(0.0, -0.593786, 0.0), (1.822785, 0.128248, 0.0), (1.271564, 0.168645, 0.0),
          (-1.271564, 0.168645, 0.0), (-1.822785, 0.128248, 0.0)]
    bodies = [nbg.MassBody(r, v, 1.0) for r, v in zip(rs, vs)]
    sim = nbg.NBodySimulation(nbg.GravitationalSystem(bodies, 1.0), (0.0, 2 * math.pi))
    desc, keep, u0, v0, u, v = _run(oracle, sim, 2 * math.pi / 200000, 200000)
    assert np.abs(u - u0).max() <= 0.01


def test_repelling_magnetic_dipoles(oracle):
    """magnetostaic_test.jl:5-32: two parallel dipoles 1 cm apart, 100 VV
    steps of 0.01 s: the speed from energy conservation within 1e-3."""
    d1, m1, rho, M, mu_4pi = 0.01, 5.0e-6, 7800.0, 1.2e6, 1.0e-7
    mm = (0.0, 0.0, M * m1 / rho)
    p1 = nbg.MagneticParticle((-d1 / 2, 0.0, 0.0), (0.0, 0.0, 0.0), m1, mm)
    p2 = nbg.MagneticParticle((d1 / 2, 0.0, 0.0), (0.0, 0.0, 0.0), m1, mm)
    system = nbg.PotentialNBodySystem([p1, p2], {"magnetostatic": nbg.MagnetostaticParameters(mu_4pi)})
    sim = nbg.NBodySimulation(system, (0.0, 1.0))
    desc, keep, u0, v0, u, v = _run(oracle, sim, 0.01, 100)
    d2 = np.linalg.norm(u[1] - u[0])
    v_expected = math.sqrt(mu_4pi * (np.dot(mm, mm) * (1 / d1 ** 3 - 1 / d2 ** 3)) / m1)
    assert abs(np.linalg.norm(v[1]) - v_expected) <= 0.001


def _ref_energies(sim, u, v):
    """The reference's energy loops (nbody_simulation_result.jl:209-212,
    281-397) in plain Python: kinetic sum(m v^2 / 2); LJ 4 eps sum_{i<j}
    (s12 - s6) with r^2 clamped to R^2 beyond the cutoff; electrostatics
    k sum_{i<j, not excluded} q_i q_j / r (or / R beyond); bonds sum k d^2 / 4
    over both ends; angles sum k (theta - theta0)^2 / 2."""
    sysm = sim.system
    bc = sim.boundary_conditions
    L = bc.L if isinstance(bc, nbg.CubicPeriodicBoundaryConditions) else None

    def dist2(i, j):
        d = [float(u[i][k]) - float(u[j][k]) for k in range(3)]
        if L is not None:
            for k in range(3):
                while d[k] >= 0.5 * L:
                    d[k] -= L
                while d[k] < -0.5 * L:
                    d[k] += L
        return d[0] ** 2 + d[1] ** 2 + d[2] ** 2

    ms = nbg.get_masses(sysm)
    out = {"kinetic": sum(float(np.dot(v[i], v[i])) * (ms[i] / 2) for i in range(len(ms)))}
    water = isinstance(sysm, nbg.WaterSPCFw)
    if water:
        lj, el = sysm.lj_parameters, sysm.e_parameters
        n = 3 * len(sysm.bodies)
        lj_idx = list(range(0, n, 3))
        qs = [sysm.qO, sysm.qH, sysm.qH] * len(sysm.bodies)
        excluded = lambda i, j: i // 3 == j // 3
    else:
        lj = sysm.potentials.get("lennard_jones")
        el = sysm.potentials.get("electrostatic")
        n = len(sysm.bodies)
        lj_idx = list(range(n))
        qs = [getattr(b, "q", 0.0) for b in sysm.bodies]
        excluded = lambda i, j: i == j
    e = 0
    if lj is not None:
        for a in range(len(lj_idx)):
            for b in range(a + 1, len(lj_idx)):
                r2 = dist2(lj_idx[a], lj_idx[b])
                if not r2 < lj.R2:
                    r2 = lj.R2
                s6 = (lj.sigma2 / r2) ** 3
                e += s6 ** 2 - s6
        out["lennard_jones"] = 4 * lj.eps * e
    if el is not None:
        e_el = 0.0
        for i in range(n):
            e_i = 0.0
            for j in range(i + 1, n):
                if not excluded(i, j):
                    r2 = dist2(i, j)
                    e_i += qs[j] / math.sqrt(r2) if r2 < el.R2 else qs[j] / el.R
            e_el += e_i * qs[i]
        out["electrostatic"] = e_el * el.k
    if water:
        p = sysm.scpfw_parameters
        eb, ea = 0, 0
        for m in range(len(sysm.bodies)):
            o, h1, h2 = 3 * m, 3 * m + 1, 3 * m + 2
            for a, b in ((o, h1), (o, h2), (h1, o), (h2, o)):
                eb += (float(np.linalg.norm(u[a] - u[b])) - p.rOH) ** 2 * p.kb
            ba, bc_ = u[h1] - u[o], u[h2] - u[o]
            ang = math.acos(float(np.dot(ba, bc_)) / (float(np.linalg.norm(ba)) * float(np.linalg.norm(bc_))))
            ea += p.ka * (ang - p.aHOH) ** 2
        out["bonds"], out["angles"] = eb / 4, ea / 2
    return out


@pytest.mark.parametrize("which", ["lj", "charges", "water"])
def test_oracle_energies_match_reference_loops(oracle, which):
    """Each energy term of the oracle against a plain restatement of the
    reference's loops, on a thermalised LJ liquid (pairs beyond the cutoff
    clamped), eight charges with a cutoff, and three water molecules."""
    if which == "lj":
        sim = S.lj_liquid(64, seed=5, jitter=0.05)
    elif which == "charges":
        sim, _ = S.charges8()
    else:
        sim, _, _ = S.water3()
    desc, keep = nbg.system_descriptor(sim)
    u0, v0 = S.state(sim)
    rng = np.random.default_rng(6)
    u = u0 + rng.normal(scale=0.01, size=u0.shape) * (0.02 if which == "water" else 1.0)
    v = v0 + rng.normal(scale=0.1, size=v0.shape)
    got = oracle.energy(desc, u, v)
    ref = _ref_energies(sim, u, v)
    for key, val in ref.items():
        assert got[key] == pytest.approx(val, rel=1e-12, abs=1e-12 * (abs(val) + 1e-300)), key


def _ref_accel(sim, u):
    """The reference's acceleration functions (basic_potentials.jl:240-433)
    in plain Python, summed per atom as soode_system! does for an NVE system
    (nbody_to_ode.jl:471-536): LJ over the LJ participants, electrostatics
    outside the exclusions, gravity, magnetic dipoles, and for water the
    bonds and the H-O-H angle."""
    sysm = sim.system
    bc = sim.boundary_conditions
    L = bc.L if isinstance(bc, nbg.CubicPeriodicBoundaryConditions) else None

    def rij(i, j):
        d = [float(u[i][k]) - float(u[j][k]) for k in range(3)]
        if L is not None:
            for k in range(3):
                while d[k] >= 0.5 * L:
                    d[k] -= L
                while d[k] < -0.5 * L:
                    d[k] += L
        return np.array(d), d[0] ** 2 + d[1] ** 2 + d[2] ** 2

    water = isinstance(sysm, nbg.WaterSPCFw)
    ms = nbg.get_masses(sysm)
    n = len(ms)
    dv = np.zeros((n, 3))
    if water:
        lj, el, grav, mag = sysm.lj_parameters, sysm.e_parameters, None, None
        lj_idx = list(range(0, n, 3))
        qs = [sysm.qO, sysm.qH, sysm.qH] * len(sysm.bodies)
        excluded = lambda i, j: i // 3 == j // 3
    else:
        pots = getattr(sysm, "potentials", {})
        lj, el = pots.get("lennard_jones"), pots.get("electrostatic")
        mag = pots.get("magnetostatic")
        grav = sysm if isinstance(sysm, nbg.GravitationalSystem) else pots.get("gravitational")
        lj_idx = list(range(n))
        qs = [getattr(b, "q", 0.0) for b in sysm.bodies]
        excluded = lambda i, j: i == j
    for i in range(n):
        if lj is not None and i in lj_idx:
            f = np.zeros(3)
            for j in lj_idx:
                if j != i:
                    d, r2 = rij(i, j)
                    if r2 < lj.R2:
                        s6 = (lj.sigma2 / r2) ** 3
                        f += (2 * s6 ** 2 - s6) / r2 * d
            dv[i] += 24 * lj.eps / ms[i] * f
        if el is not None:
            f = np.zeros(3)
            for j in range(n):
                if not excluded(i, j):
                    d, r2 = rij(i, j)
                    if r2 < el.R2:
                        f += qs[j] / (math.sqrt(r2) * r2) * d
            dv[i] += el.k * qs[i] / ms[i] * f
        if grav is not None:
            for j in range(n):
                if j != i:
                    d = u[i] - u[j]
                    dv[i] += -grav.G * sysm.bodies[j].m / np.linalg.norm(d) ** 3 * d
        if mag is not None:
            f = np.zeros(3)
            mi = np.asarray(sysm.bodies[i].mm, dtype=float)
            for j in range(n):
                if j != i:
                    mj = np.asarray(sysm.bodies[j].mm, dtype=float)
                    d = u[i] - u[j]
                    r = d / np.linalg.norm(d)
                    mir, mij = np.dot(mi, r), np.dot(mj, r)
                    f += (mi * mij + mj * mir + r * np.dot(mi, mj) - 5 * r * mir * mij) / np.dot(d, d) ** 2
            dv[i] += 3 * mag.mu_4pi / sysm.bodies[i].m * f
    if water:
        p = sysm.scpfw_parameters
        for m in range(len(sysm.bodies)):
            o, h1, h2 = 3 * m, 3 * m + 1, 3 * m + 2
            for i, nbrs in ((o, (h1, h2)), (h1, (o,)), (h2, (o,))):
                for j in nbrs:
                    d = u[i] - u[j]
                    r = np.linalg.norm(d)
                    dv[i] += -(r - p.rOH) * p.kb / r * d / ms[i]
            rba, rbc, rcb = u[h1] - u[o], u[h2] - u[o], u[o] - u[h2]
            x = np.cross(rba, rbc)
            pa = np.cross(rba, x)
            pa = pa / np.linalg.norm(pa)
            pc = np.cross(rcb, x)
            pc = pc / np.linalg.norm(pc)
            c = min(1.0, max(-1.0, float(np.dot(rba, rbc)) / (np.linalg.norm(rba) * np.linalg.norm(rbc))))
            force = -p.ka * (math.acos(c) - p.aHOH)
            fa = pa * force / np.linalg.norm(rba)
            fc = pc * force / np.linalg.norm(rbc)
            dv[h1] += fa / ms[h1]
            dv[o] += -(fa + fc) / ms[o]
            dv[h2] += fc / ms[h2]
    return dv


@pytest.mark.parametrize("which", ["lj", "charges", "gravity", "magnetic", "water"])
def test_oracle_accelerations_match_reference_loops(oracle, which):
    """The oracle's right-hand side against a plain restatement of the
    reference's acceleration functions, to 1e-10 of the largest component."""
    rng = np.random.default_rng(8)
    if which == "lj":
        sim = S.lj_liquid(64, seed=5, jitter=0.05)
    elif which == "charges":
        sim, _ = S.charges8()
    elif which == "gravity":
        sim = S.plummer(32)
    elif which == "magnetic":
        bodies = [nbg.MagneticParticle(rng.uniform(-1, 1, 3), (0, 0, 0), 1.0 + rng.random(), rng.normal(size=3))
                  for _ in range(6)]
        sim = nbg.NBodySimulation(nbg.PotentialNBodySystem(bodies, {"magnetostatic": nbg.MagnetostaticParameters(1.0)}),
                                  (0.0, 1.0))
    else:
        sim, _, _ = S.water3()
    desc, keep = nbg.system_descriptor(sim)
    u0, v0 = S.state(sim)
    u = u0 + rng.normal(scale=0.01 if which != "water" else 0.002, size=u0.shape)
    dv, _ = oracle.accel(desc, v0, u)
    ref = _ref_accel(sim, u)
    scale = np.abs(ref).max()
    assert scale > 0
    assert np.abs(dv[: len(ref)] - ref).max() <= 1e-10 * scale


@pytest.mark.parametrize("which", ["lj_berendsen", "lj_nosehoover", "water_berendsen", "water_nosehoover"])
def test_oracle_thermostat_terms_match_reference(oracle, which):
    """The simultaneous thermostat terms of soode_system! against the
    reference (thermostats.jl:76-128, data nbody_to_ode.jl:392-433):
    T = sum m v^2 / (kb (3N - Nc)) (no 1/2; Nc = 2 per water molecule);
    Berendsen dv += gamma (T0 / T - 1) v, gamma = 0.5 / tau; Nose-Hoover
    dv -= zeta v with zeta = u[3N+1], dv of the extra column 0, and
    v[3N+1] = tau^-2 (T / T0 - (ndf + 1) / ndf)."""
    rng = np.random.default_rng(9)
    T0, tau = (1.0, 0.3) if which.startswith("lj") else (300.0, 0.1)
    th = (nbg.BerendsenThermostat(T0, tau) if which.endswith("berendsen") else nbg.NoseHooverThermostat(T0, tau))
    if which.startswith("lj"):
        sim = S.lj_liquid(64, seed=5, jitter=0.05, thermostat=th)
        kb, N, Nc = 1.0, 64, 0
    else:
        sim = S.water_box(8, seed=2, thermostat=th)
        kb, N, Nc = S.KB_KJ, 24, 16
    desc, keep = nbg.system_descriptor(sim)
    u0, v0 = S.state(sim)
    u = u0.copy()
    u[:N] += rng.normal(scale=0.002, size=(N, 3))
    v = v0 + rng.normal(scale=0.05, size=v0.shape)
    nh = which.endswith("nosehoover")
    if nh:
        assert u.shape[0] == N + 1
        u[N] = (0.37, 0.0, 0.0)  # zeta
        v[N] = (0.0, 0.0, 0.0)
    dv, v_out = oracle.accel(desc, v.copy(), u)
    ms = nbg.get_masses(sim.system)
    forces = _ref_accel(sim, u[:N])
    T = float(sum(ms[i] * np.dot(v[i], v[i]) for i in range(N))) / (kb * (3 * N - Nc))
    if nh:
        zeta = u[N][0]
        ref = np.vstack([forces - zeta * v[:N], np.zeros((1, 3))])
        ndf = 3 * N - Nc
        assert v_out[N][0] == pytest.approx(tau ** -2 * (T / T0 - (ndf + 1) / ndf), rel=1e-12)
    else:
        ref = forces + (0.5 / tau) * (T0 / T - 1) * v[:N]
    assert np.abs(dv - ref).max() <= 1e-10 * np.abs(ref).max()


def test_oracle_langevin_drift_matches_reference():
    """SDEProblem for a potential system (nbody_to_ode.jl:567-598): the drift
    is du = v, dv = a(u) - gamma v, and Euler-Maruyama steps X' = X + dt f(X)
    + g dW. At T = 0 the noise amplitude sqrt(2 gamma kb T / m) vanishes, so
    one oracle step must equal the drift step exactly as restated here."""
    import __graft_entry__ as g
    oracle = g.load_oracle()
    gamma, dt = 0.7, 0.004
    sim = S.lj_liquid(64, seed=5, jitter=0.05, thermostat=nbg.LangevinThermostat(0.0, gamma))
    desc, keep = nbg.system_descriptor(sim)
    u0, v0 = S.state(sim)
    u1, v1 = oracle.run(desc, u0, v0, dt, 1)
    a = _ref_accel(sim, u0)
    assert np.abs(u1 - (u0 + dt * v0)).max() <= 1e-14 * np.abs(u0).max()
    ref_v = v0 + dt * (a - gamma * v0)
    assert np.abs(v1 - ref_v).max() <= 1e-10 * np.abs(ref_v).max()


def _adaptive(oracle, sim):
    """run_simulation(sim)'s host adaptive integration (simulation.py
    _adaptive_run) with the oracle's right-hand side in place of nbg_accel."""
    desc, keep = nbg.system_descriptor(sim)
    u0, v0 = S.state(sim)
    rhs = lambda v, u, t: oracle.accel(desc, v, u, t)[0]
    return nbg.simulation._adaptive_run(rhs, u0, v0, sim.tspan, 1e-6, 1e-3, True)


def test_default_adaptive_run_closes_the_figure_eight(oracle):
    """gravitational_test.jl:8-24: run_simulation(simulation) with the default
    adaptive method returns the figure-eight to its start after 2 pi within
    0.1; the saved times are the accepted steps from 0 to 2 pi."""
    t, tu, tv, nacc = _adaptive(oracle, S.figure8())
    assert t[0] == 0.0 and t[-1] == pytest.approx(2 * math.pi) and nacc == len(t) - 1 > 10
    assert np.abs(tu[-1] - tu[0]).max() <= 0.1


def test_adaptive_frames_feed_msd_and_interpolation(oracle):
    """The adaptive path's frames are one (frames, cols, 3) array like the
    fused path's, so msd (nbody_simulation_result.jl:730-783) and the
    interpolation between saved times work on its result."""
    sim = S.figure8()
    t, tu, tv, nacc = _adaptive(oracle, sim)
    sr = nbg.SimulationResult(nbg.simulation.Solution(t, tu, tv, nacc), sim)
    assert sr.solution.u.shape == (len(t), 3, 3)
    ts, m = nbg.msd(sr)
    U = np.stack(tu)
    ref = ((U - U[0]) ** 2).sum(axis=2).mean(axis=1)
    assert np.array_equal(ts, t) and m[0] == 0.0 and np.allclose(m, ref, rtol=0, atol=0)
    mid = 0.5 * (t[3] + t[4])
    p = nbg.get_position(sr, mid)
    assert p.shape == (3, 3) and np.all(np.isfinite(p))


def test_default_adaptive_run_closes_the_charge_orbit(oracle):
    """electrostatics_test.jl:7-29, with run_simulation(simulation)'s default
    adaptive method: back at the start after one period within 0.1 r."""
    k, r, q1, q2, m1, m2 = 9.0e9, 100.0, 1.0e-3, -1.0e-3, 100.0, 0.1
    v2 = math.sqrt(abs(k * q1 * q2 / m2 / r))
    p1 = nbg.ChargedParticle((0.0, 0.0, 0.0), (0.0, 0.0, 0.0), m1, q1)
    p2 = nbg.ChargedParticle((r, 0.0, 0.0), (0.0, v2, 0.0), m2, q2)
    sim = nbg.NBodySimulation(nbg.ChargedParticles([p1, p2], k), (0.0, 2 * math.pi * r / v2))
    t, tu, tv, nacc = _adaptive(oracle, sim)
    assert np.abs(tu[-1] - tu[0]).max() <= 0.1 * r


def test_default_adaptive_run_refuses_stateful_thermostats():
    """Nose-Hoover writes zeta into v inside the right-hand side, Andersen is
    a callback and Langevin an SDE: run_simulation(sim) without dt refuses
    them (NBG_ERR_UNSUPPORTED) before touching the GPU."""
    for th in (nbg.NoseHooverThermostat(1.0, 0.1), nbg.AndersenThermostat(1.0, 0.1), nbg.LangevinThermostat(1.0, 1.0)):
        sim = S.lj_liquid(64, seed=1, thermostat=th)
        with pytest.raises(nbg.EngineError) as e:
            nbg.run_simulation(sim)
        assert e.value.status == -6
