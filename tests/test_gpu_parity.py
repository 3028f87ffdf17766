"""GPU engine (libnbg.so through the C ABI) against the FP64 oracle on the
same seeded inputs: forces within the relative-RMSE tolerance of 1e-5, the
cutoff pair sets bit for bit, energies, thermostat terms and trajectories."""
import math
import os

import numpy as np
import pytest

import systems as S

nbg = S.nbg
pytestmark = pytest.mark.gpu

FORCE_TOL = 1e-5  # relative RMSE of accelerations vs the FP64 oracle


def _accel_pair(gpu, oracle, sim, perturb=0.0, seed=0):
    desc, keep = nbg.system_descriptor(sim)
    u, v = S.state(sim)
    if perturb:
        rng = np.random.default_rng(seed)
        n = desc.n
        u = u.copy()
        u[:n] += rng.uniform(-perturb, perturb, size=(n, 3))
    eng = nbg.Engine(desc, 0)
    a_gpu = eng.accel(v.copy(), u)
    a_ref, _ = oracle.accel(desc, v, u)
    return eng, desc, keep, u, v, a_gpu, a_ref


@pytest.mark.parametrize("flags", [0, nbg._abi.NBG_FLAG_GRAV_PLAIN])
def test_gravity_forces(gpu, oracle, flags):
    sim = S.plummer(3000, seed=5, flags=flags)
    eng, desc, keep, u, v, ag, ar = _accel_pair(gpu, oracle, sim)
    err = S.rel_rmse(ag, ar)
    print(f"gravity {'plain' if flags else 'compensated'} rel RMSE {err:.3e}")
    if not flags:
        assert err <= FORCE_TOL
    else:
        assert err <= 1e-3
    # Newton's third law in the sum: total force ~ 0
    m = np.asarray(keep[0])
    assert np.abs((m[:, None] * ag).sum(axis=0)).max() <= 1e-6 * np.abs(m[:, None] * ag).sum()


@pytest.mark.parametrize("flags", [0, nbg._abi.NBG_FLAG_GRAV_PLAIN])
def test_gravity_forces_unequal_masses(gpu, oracle, flags):
    """Unequal masses keep m_j inside the pair loop (equal masses apply G m
    once, in the reduction): both forms against the oracle."""
    sim = S.plummer(2500, seed=9, flags=flags, mass_spread=0.5)
    eng, desc, keep, u, v, ag, ar = _accel_pair(gpu, oracle, sim)
    err = S.rel_rmse(ag, ar)
    assert err <= (FORCE_TOL if not flags else 1e-3), err
    m = np.asarray(keep[0])
    assert np.abs((m[:, None] * ag).sum(axis=0)).max() <= 1e-6 * np.abs(m[:, None] * ag).sum()


def test_gravity_tile_edges(gpu, oracle):
    """N not a multiple of the 256-body tile: padding bodies contribute nothing."""
    for n in (3, 257, 511, 1000):
        sim = S.plummer(n, seed=n)
        eng, desc, keep, u, v, ag, ar = _accel_pair(gpu, oracle, sim)
        assert S.rel_rmse(ag, ar) <= FORCE_TOL, n
        eng.close()


@pytest.mark.parametrize("flags", [0, nbg._abi.NBG_FLAG_ALL_PAIRS])
def test_lj_forces_and_pair_set(gpu, oracle, flags):
    sim = S.lj_liquid(1000, seed=2, jitter=0.15, flags=flags)
    eng, desc, keep, u, v, ag, ar = _accel_pair(gpu, oracle, sim)
    assert S.rel_rmse(ag, ar) <= FORCE_TOL
    pg = eng.pair_list(u, nbg._abi.NBG_POT_LJ)
    po = oracle.pair_list(desc, u, nbg._abi.NBG_POT_LJ)
    assert pg.shape == po.shape and np.array_equal(pg, po)


@pytest.mark.parametrize("lanes", [None, "4", "32"])
def test_lj_pair_set_at_cutoff_boundary(gpu, oracle, lanes):
    """Pairs placed within a few ulps of r = R: the FP64 re-check decides
    (the split-position classification of a thread per atom, and the
    fixed-point one of the lanes-per-atom kernel)."""
    R = 2.5
    L = 10.0
    eps = np.finfo(np.float64).eps
    pos = []
    for k, d in enumerate([R * (1 - 4 * eps), R, R * (1 + 4 * eps), R * (1 - 1e-7), R * (1 + 1e-7)]):
        base = np.array([1.0 + 1.9 * k, 0.5 + 1.9 * k, 2.0])
        pos += [base, base + np.array([d, 0.0, 0.0])]
    # across the periodic boundary as well
    pos += [np.array([0.2, 7.0, 7.0]), np.array([0.2 + L - R, 7.0, 7.0])]
    pos = np.array(pos)
    bodies = [nbg.MassBody(p, (0, 0, 0), 1.0) for p in pos]
    system = nbg.PotentialNBodySystem(bodies, {"lennard_jones": nbg.LennardJonesParameters(1.0, 1.0, R)})
    sim = nbg.NBodySimulation(system, (0.0, 1.0), nbg.CubicPeriodicBoundaryConditions(L), kb=1.0, skin=0.3)
    desc, keep = nbg.system_descriptor(sim)
    u, v = S.state(sim)
    if lanes:
        os.environ["NBG_LIST_LPA"] = lanes
    try:
        eng = nbg.Engine(desc, 0)
    finally:
        os.environ.pop("NBG_LIST_LPA", None)
    form = eng.force_form()
    assert form == ((int(lanes), True) if lanes else (1, False)), form
    pg = eng.pair_list(u, nbg._abi.NBG_POT_LJ)
    po = oracle.pair_list(desc, u, nbg._abi.NBG_POT_LJ)
    assert np.array_equal(pg, po)
    # the forces count exactly those pairs
    ag = eng.accel(v.copy(), u)
    ar, _ = oracle.accel(desc, v.copy(), u)
    assert np.abs(ag - ar).max() <= 1e-5 * np.abs(ar).max()


def test_coulomb_unbounded_forces(gpu, oracle):
    rng = np.random.default_rng(4)
    n = 300
    bodies = [nbg.ChargedParticle(rng.uniform(-1, 1, 3), (0, 0, 0), rng.uniform(0.5, 2), rng.choice([-1.0, 1.0]))
              for _ in range(n)]
    sim = nbg.NBodySimulation(nbg.ChargedParticles(bodies, 1.0), (0.0, 1.0))
    eng, desc, keep, u, v, ag, ar = _accel_pair(gpu, oracle, sim)
    assert S.rel_rmse(ag, ar) <= FORCE_TOL


def test_lj_plus_coulomb_cubic(gpu, oracle):
    """Both cutoff potentials on one system (distinct cutoffs) on the list path."""
    pos, vel, L = nbg.workloads.lj_argon_lattice(1000, seed=9, jitter=0.1)
    rng = np.random.default_rng(9)
    bodies = [nbg.ChargedParticle(pos[i], vel[i], 1.0, rng.choice([-0.5, 0.5])) for i in range(len(pos))]
    system = nbg.PotentialNBodySystem(bodies, {"lennard_jones": nbg.LennardJonesParameters(1.0, 1.0, 2.5),
                                               "electrostatic": nbg.ElectrostaticParameters(1.0, 3.0)})
    sim = nbg.NBodySimulation(system, (0.0, 1.0), nbg.CubicPeriodicBoundaryConditions(L), kb=1.0, skin=0.3)
    eng, desc, keep, u, v, ag, ar = _accel_pair(gpu, oracle, sim)
    assert S.rel_rmse(ag, ar) <= FORCE_TOL
    for which in (nbg._abi.NBG_POT_LJ, nbg._abi.NBG_POT_EL):
        assert np.array_equal(eng.pair_list(u, which), oracle.pair_list(desc, u, which))


def test_magnetic_dipoles(gpu, oracle):
    rng = np.random.default_rng(5)
    bodies = [nbg.MagneticParticle(rng.uniform(-1, 1, 3), (0, 0, 0), 1.0, rng.normal(size=3)) for _ in range(64)]
    system = nbg.PotentialNBodySystem(bodies, {"magnetostatic": nbg.MagnetostaticParameters(1.0)})
    sim = nbg.NBodySimulation(system, (0.0, 1.0))
    eng, desc, keep, u, v, ag, ar = _accel_pair(gpu, oracle, sim)
    assert S.rel_rmse(ag, ar) <= FORCE_TOL


@pytest.mark.parametrize("n_mol", [3, 216, 1000])
def test_water_forces_and_pair_sets(gpu, oracle, n_mol):
    """SPC/Fw: O-O LJ, molecule-excluded electrostatics, bonds, angles (all-pairs
    path for small boxes, Verlet-list path for 1000 molecules)."""
    if n_mol == 3:
        sim, _, _ = S.water3()
    else:
        sim = S.water_box(n_mol, seed=n_mol)
    eng, desc, keep, u, v, ag, ar = _accel_pair(gpu, oracle, sim)
    assert S.rel_rmse(ag, ar) <= FORCE_TOL
    for which in (nbg._abi.NBG_POT_LJ, nbg._abi.NBG_POT_EL):
        assert np.array_equal(eng.pair_list(u, which), oracle.pair_list(desc, u, which))


def test_reaction_field_eps1_equals_truncated_coulomb(gpu):
    """eps_rf = 1 is the reference's truncated Coulomb; eps_rf > 1 adds the
    2 k_rf r term."""
    s1 = S.water_box(1000, seed=1, eps_rf=1.0)
    s2 = S.water_box(1000, seed=1, eps_rf=78.0)
    d1, k1 = nbg.system_descriptor(s1)
    d2, k2 = nbg.system_descriptor(s2)
    u, v = S.state(s1)
    a1 = nbg.Engine(d1, 0).accel(v.copy(), u)
    a2 = nbg.Engine(d2, 0).accel(v.copy(), u)
    assert S.rel_rmse(a2, a1) > 1e-4


@pytest.mark.parametrize("kind", ["berendsen", "nosehoover"])
def test_thermostat_rhs(gpu, oracle, kind):
    th = nbg.BerendsenThermostat(0.8, 0.1) if kind == "berendsen" else nbg.NoseHooverThermostat(0.8, 0.1)
    sim = S.lj_liquid(1000, seed=3, jitter=0.1, thermostat=th)
    desc, keep = nbg.system_descriptor(sim)
    u, v = S.state(sim)
    if kind == "nosehoover":
        u[-1, 0] = 0.37  # zeta
    eng = nbg.Engine(desc, 0)
    vg = v.copy()
    ag = eng.accel(vg, u)
    ar, vr = oracle.accel(desc, v, u)
    assert S.rel_rmse(ag, ar) <= FORCE_TOL
    if kind == "nosehoover":
        assert vg[-1, 0] == pytest.approx(vr[-1, 0], rel=1e-12)
        assert np.all(ag[-1] == 0)


def test_energies_match_oracle(gpu, oracle):
    for sim in (S.lj_liquid(1000, seed=4, jitter=0.1), S.water_box(216, seed=2), S.plummer(2000, seed=1),
                S.water3()[0], S.charges8()[0]):
        desc, keep = nbg.system_descriptor(sim)
        u, v = S.state(sim)
        eg = nbg.Engine(desc, 0).energy(u, v)
        eo = oracle.energy(desc, u, v)
        scale = sum(abs(eo[k]) for k in ("kinetic", "lennard_jones", "electrostatic", "bonds", "angles", "gravity"))
        for k in ("kinetic", "lennard_jones", "electrostatic", "bonds", "angles", "gravity"):
            assert eg[k] == pytest.approx(eo[k], rel=1e-11, abs=1e-13 * scale), k
        assert eg["temperature"] == pytest.approx(eo["temperature"], rel=1e-12)


@pytest.mark.parametrize("case", ["lj_list", "lj_berendsen", "lj_nosehoover", "water_list", "gravity"])
def test_short_trajectories(gpu, oracle, case):
    """A few velocity-Verlet steps on the GPU track the FP64 oracle (FP32 pair
    forces, FP64 integration)."""
    if case == "lj_list":
        sim, dt, n, tol = S.lj_liquid(1000, seed=5), 0.005, 25, 1e-8
    elif case == "lj_berendsen":
        sim, dt, n, tol = S.lj_liquid(1000, seed=5, thermostat=nbg.BerendsenThermostat(1.5, 0.05)), 0.005, 25, 1e-8
    elif case == "lj_nosehoover":
        sim, dt, n, tol = S.lj_liquid(1000, seed=5, thermostat=nbg.NoseHooverThermostat(1.5, 0.05)), 0.005, 25, 1e-8
    elif case == "water_list":
        sim, dt, n, tol = S.water_box(1000, seed=6), 0.0005, 20, 1e-8
    else:
        sim, dt, n, tol = S.plummer(2048, seed=6), 1e-3, 20, 1e-8
    desc, keep = nbg.system_descriptor(sim)
    u, v = S.state(sim)
    eng = nbg.Engine(desc, 0)
    ug, vg, _, _, stats = eng.run(u, v, dt, n, 0, save_trajectory=False)
    uo, vo = oracle.run(desc, u, v, dt, n)
    na = int(desc.n)
    scale = np.abs(uo[:na]).max()
    assert np.abs(ug[:na] - uo[:na]).max() <= tol * max(scale, 1.0), np.abs(ug[:na] - uo[:na]).max()
    if len(uo) > na:
        # the Nose-Hoover variable integrates the temperature error of FP32
        # pair forces: relative agreement at that level
        assert abs(ug[na, 0] - uo[na, 0]) <= 1e-7 * max(abs(uo[na, 0]), 1.0), (ug[na], uo[na])
    assert stats.kernel_launches > 0


def test_langevin_em_one_step(gpu, oracle):
    """Euler-Maruyama with the same Philox draws (FP32 Box-Muller on the GPU)."""
    sim = S.lj_liquid(1000, seed=6, thermostat=nbg.LangevinThermostat(1.0, 1.0))
    desc, keep = nbg.system_descriptor(sim)
    u, v = S.state(sim)
    ug, vg, _, _, _ = nbg.Engine(desc, 0).run(u, v, 0.005, 1, 0, save_trajectory=False)
    uo, vo = oracle.run(desc, u, v, 0.005, 1)
    assert np.abs(ug - uo).max() <= 1e-12
    assert np.abs(vg - vo).max() <= 1e-5 * np.abs(vo).max()


def test_baoab_one_step_and_batch(gpu, oracle):
    """BAOAB Langevin steps with the same Philox draws (FP32 Box-Muller on the
    GPU), single system and a batch of uneven replicas."""
    sim = S.lj_liquid(1000, seed=6, thermostat=nbg.LangevinThermostat(1.0, 1.0),
                      flags=nbg._abi.NBG_FLAG_LANGEVIN_BAOAB)
    desc, keep = nbg.system_descriptor(sim)
    u, v = S.state(sim)
    ug, vg, _, _, _ = nbg.Engine(desc, 0).run(u, v, 0.005, 3, 0, save_trajectory=False)
    uo, vo = oracle.run(desc, u, v, 0.005, 3)
    assert np.abs(ug - uo).max() <= 1e-6 * desc.box[0]
    assert np.abs(vg - vo).max() <= 1e-5 * np.abs(vo).max()
    sizes = [256, 1000, 1500]
    descs, keep, us, vs = _ensemble(nbg, sizes, lambda r: nbg.LangevinThermostat(0.9 + 0.3 * r, 1.0))
    for d in descs:
        d.flags |= nbg._abi.NBG_FLAG_LANGEVIN_BAOAB
    ug, vg, _, _, _ = nbg.Engine(descs, 0).run(np.concatenate(us), np.concatenate(vs), 0.005, 1, 0,
                                               save_trajectory=False)
    off = 0
    for r, n in enumerate(sizes):
        uo, vo = oracle.run(descs[r], us[r], vs[r], 0.005, 1)
        assert np.abs(ug[off:off + n] - uo).max() <= 1e-6 * descs[r].box[0]
        assert np.abs(vg[off:off + n] - vo).max() <= 1e-5 * np.abs(vo).max()
        off += n


def test_andersen_one_step(gpu, oracle):
    sim = S.lj_liquid(1000, seed=7, thermostat=nbg.AndersenThermostat(1.0, 20.0))
    desc, keep = nbg.system_descriptor(sim)
    u, v = S.state(sim)
    ug, vg, _, _, _ = nbg.Engine(desc, 0).run(u, v, 0.005, 1, 0, save_trajectory=False)
    uo, vo = oracle.run(desc, u, v, 0.005, 1)
    # atoms that collided got their velocity redrawn: FP64 normals on both
    # sides; the rest went through the kick with FP32 pair forces
    sim0 = S.lj_liquid(1000, seed=7)
    d0, k0 = nbg.system_descriptor(sim0)
    _, v_nocoll = oracle.run(d0, u, v, 0.005, 1)
    changed = np.any(vo != v_nocoll, axis=1)
    assert changed.sum() > 20
    assert np.abs(vg[changed] - vo[changed]).max() <= 1e-12 * np.abs(vo).max()
    assert np.abs(vg[~changed] - vo[~changed]).max() <= 1e-6 * np.abs(vo).max()


def test_nonfinite_state_reported(gpu):
    """NaN positions end the call with NBG_ERR_NONFINITE; the context stays usable."""
    sim = S.plummer(512, seed=1)
    desc, keep = nbg.system_descriptor(sim)
    u, v = S.state(sim)
    eng = nbg.Engine(desc, 0)
    bad = u.copy()
    bad[3, 0] = np.nan
    with pytest.raises(nbg.EngineError) as ei:
        eng.run(bad, v, 1e-3, 2, 0, save_trajectory=False)
    assert ei.value.status == -4
    eng.run(u, v, 1e-3, 2, 0, save_trajectory=False)


def test_capacity_regrowth(gpu, oracle):
    """A dense cluster overflows the initial cell and neighbour capacities;
    the engine grows them and reruns, matching the oracle."""
    pos, vel, L = nbg.workloads.lj_argon_lattice(1000, seed=8, jitter=0.1)
    pos[:200] = pos[:200] * 0.35 + 0.5  # compress a fifth of the atoms into one corner
    bodies = [nbg.MassBody(pos[i], vel[i] * 0.0, 1.0) for i in range(len(pos))]
    system = nbg.PotentialNBodySystem(bodies, {"lennard_jones": nbg.LennardJonesParameters(1.0, 0.5, 2.5)})
    sim = nbg.NBodySimulation(system, (0.0, 1.0), nbg.CubicPeriodicBoundaryConditions(L), kb=1.0, skin=0.3)
    eng, desc, keep, u, v, ag, ar = _accel_pair(gpu, oracle, sim)
    assert S.rel_rmse(ag, ar) <= FORCE_TOL


def _ensemble(nbg, sizes, thermostat_of):
    descs, keep, us, vs = [], [], [], []
    for r, n in enumerate(sizes):
        pos, vel, L = nbg.workloads.lj_argon_lattice(n, seed=40 + r, jitter=0.1, T=0.8 + 0.2 * r)
        d, k = nbg.lennard_jones_descriptor(np.ones(n), L, thermostat=thermostat_of(r), seed=77 + r, skin=0.3)
        descs.append(d)
        keep.append(k)
        us.append(pos)
        vs.append(vel)
    return descs, keep, us, vs


def test_batch_langevin_matches_oracle(gpu, oracle):
    """Uneven replicas (one of them a single cell) in one context: one
    Euler-Maruyama step per replica against the oracle per replica."""
    sizes = [256, 1000, 1500]
    descs, keep, us, vs = _ensemble(nbg, sizes, lambda r: nbg.LangevinThermostat(0.9 + 0.3 * r, 1.0))
    eng = nbg.Engine(descs, 0)
    ug, vg, _, _, _ = eng.run(np.concatenate(us), np.concatenate(vs), 0.005, 1, 0, save_trajectory=False)
    off = 0
    for r, n in enumerate(sizes):
        uo, vo = oracle.run(descs[r], us[r], vs[r], 0.005, 1)
        assert np.abs(ug[off:off + n] - uo).max() <= 1e-12
        assert np.abs(vg[off:off + n] - vo).max() <= 1e-5 * np.abs(vo).max()
        off += n


def test_batch_nve_matches_single_contexts(gpu):
    """The same replicas without thermostat: a batch of 3 gives the
    accelerations of 3 separate contexts (replicas do not interact), and short
    velocity-Verlet runs agree to the FP32 summation-order level."""
    sizes = [256, 1000, 1500]
    descs, keep, us, vs = _ensemble(nbg, sizes, lambda r: None)
    eng = nbg.Engine(descs, 0)
    U, V = np.concatenate(us), np.concatenate(vs)
    ab = eng.accel(V.copy(), U)
    ug, vg, _, _, _ = eng.run(U, V, 0.005, 10, 0, save_trajectory=False)
    off = 0
    for r, n in enumerate(sizes):
        single = nbg.Engine(descs[r], 0)
        a1 = single.accel(vs[r].copy(), us[r])
        assert S.rel_rmse(ab[off:off + n], a1) <= 1e-6
        u1, v1, _, _, _ = single.run(us[r], vs[r], 0.005, 10, 0, save_trajectory=False)
        assert np.abs(ug[off:off + n] - u1).max() <= 1e-7 * descs[r].box[0]
        off += n


def test_batch_many_cells_matches_oracle(gpu, oracle):
    """A batch with at least two cells per SM, which the warp-per-cell list
    builder serves (a single-cell replica among them): accelerations per
    replica against the oracle, and 40 velocity-Verlet steps (list rebuilds
    by displacement included) against separate contexts, whose fewer cells
    take the per-atom builders with the same candidate order."""
    import torch
    sizes = [256, 4000, 3000, 2000, 1200]
    descs, keep, us, vs = _ensemble(nbg, sizes, lambda r: None)
    cells = sum(max(int(d.box[0] // (d.lj_cutoff + d.skin)), 1) ** 3 if d.box[0] >= 3 * (d.lj_cutoff + d.skin) else 1
                for d in descs)
    assert cells >= 2 * torch.cuda.get_device_properties(0).multi_processor_count, cells
    eng = nbg.Engine(descs, 0)
    U, V = np.concatenate(us), np.concatenate(vs)
    ab = eng.accel(V.copy(), U)
    ug, vg, _, _, _ = eng.run(U, V, 0.005, 40, 0, save_trajectory=False)
    off = 0
    for r, n in enumerate(sizes):
        ao, _ = oracle.accel(descs[r], vs[r], us[r])
        assert S.rel_rmse(ab[off:off + n], ao) <= FORCE_TOL, r
        u1, v1, _, _, _ = nbg.Engine(descs[r], 0).run(us[r], vs[r], 0.005, 40, 0, save_trajectory=False)
        # FP32 pair sums in another order (the batch's lists): rounding apart
        assert np.abs(ug[off:off + n] - u1).max() <= 2e-7 * descs[r].box[0], r
        off += n


def _engine_without_cluster(desc):
    """An engine on the graph step loop (NBG_NO_CLUSTER is read at creation)."""
    import os
    os.environ["NBG_NO_CLUSTER"] = "1"
    try:
        return nbg.Engine(desc, 0)
    finally:
        del os.environ["NBG_NO_CLUSTER"]


@pytest.mark.parametrize("n", [1000, 512])
def test_cluster_step_loop(gpu, oracle, n):
    """Small NVE systems run velocity Verlet as one persistent cluster launch
    per chunk (positions in distributed shared memory, lists per CTA):
    - 20 steps against the oracle, within 1e-8 of the box or 3x the graph
      step loop's own deviation on the same system;
    - 60 steps in launches of 20 (trajectory frames; lists rebuilt in each)
      against the graph step loop on the same system. The lists hold the same
      pairs in another order, so the two differ by FP32 summation order;
    - 600 steps conserve energy as well as the graph loop does. (Trajectories
      that long are not compared: a truncated LJ force jumps at the cutoff,
      so rounding-level differences move pair crossings by a step and grow
      fast.)"""
    sim = S.lj_liquid(n, seed=12, jitter=0.1)
    desc, keep = nbg.system_descriptor(sim)
    u, v = S.state(sim)
    L = desc.box[0]
    eng = nbg.Engine(desc, 0)
    assert eng.cluster_shape() is not None
    ref = _engine_without_cluster(desc)
    assert ref.cluster_shape() is None
    ug, vg, _, _, _ = eng.run(u, v, 0.005, 20, 0, save_trajectory=False)
    ur, vr, _, _, _ = ref.run(u, v, 0.005, 20, 0, save_trajectory=False)
    uo, vo = oracle.run(desc, u, v, 0.005, 20)
    err, err_ref = np.abs(ug - uo).max(), np.abs(ur - uo).max()
    assert err <= max(1e-8 * L, 3.0 * err_ref), (err, err_ref)
    assert np.abs(vg - vo).max() <= max(1e-6 * np.abs(vo).max(), 3.0 * np.abs(vr - vo).max())
    ug, vg, tug, _, _ = eng.run(u, v, 0.005, 60, 20)
    ur, vr, tur, _, _ = ref.run(u, v, 0.005, 60, 20)
    assert np.abs(tug - tur).max() <= 1e-7 * L
    assert np.abs(vg - vr).max() <= 1e-5 * np.abs(vr).max()
    ug, vg, _, _, _ = eng.run(u, v, 0.005, 600, 0, save_trajectory=False)
    ur, vr, _, _, _ = ref.run(u, v, 0.005, 600, 0, save_trajectory=False)
    e0 = eng.energy(u, v)["total"]
    d_cl = abs(eng.energy(ug, vg)["total"] - e0)
    d_ref = abs(ref.energy(ur, vr)["total"] - e0)
    assert d_cl <= 3.0 * d_ref + 1e-5 * abs(e0), (d_cl, d_ref)


def test_cluster_step_loop_list_regrowth(gpu, oracle):
    """A compressed region overflows the cluster path's list capacity: the
    chunk is undone, the lists grow (the cluster plan follows the new
    capacity) and the chunk runs again, matching the oracle as closely as the
    graph step loop does."""
    pos, vel, L = nbg.workloads.lj_argon_lattice(1000, seed=8, jitter=0.05)
    sel = slice(0, 300)
    ctr = pos[sel].mean(axis=0)
    pos[sel] = ctr + 0.8 * (pos[sel] - ctr)  # density ~1.6 there: ~150 neighbours
    bodies = [nbg.MassBody(pos[i], vel[i], 1.0) for i in range(len(pos))]
    system = nbg.PotentialNBodySystem(bodies, {"lennard_jones": nbg.LennardJonesParameters(1.0, 1.0, 2.5)})
    sim = nbg.NBodySimulation(system, (0.0, 1.0), nbg.CubicPeriodicBoundaryConditions(L), kb=1.0, skin=0.3)
    desc, keep = nbg.system_descriptor(sim)
    u, v = S.state(sim)
    eng = nbg.Engine(desc, 0)
    assert eng.cluster_shape() is not None
    ref = _engine_without_cluster(desc)
    ug, vg, _, _, _ = eng.run(u, v, 0.002, 20, 0, save_trajectory=False)
    ur, vr, _, _, _ = ref.run(u, v, 0.002, 20, 0, save_trajectory=False)
    uo, vo = oracle.run(desc, u, v, 0.002, 20)
    err, err_ref = np.abs(ug - uo).max(), np.abs(ur - uo).max()
    assert err <= max(1e-8 * L, 3.0 * err_ref), (err, err_ref)
    assert eng.cluster_shape() is not None  # still on the cluster path, with the larger lists


@pytest.mark.parametrize("drop", ["last", "5"])
def test_cluster_loop_timeout_is_reported_and_recovers(gpu, oracle, drop):
    """The persistent cluster loop's bounded waits: with a host-set test flag
    (NBG_TEST_CLUSTER_DROP, read at creation, used by the first launch only)
    no CTA sends its positions in one step, so every receiver's wait runs
    out with no copy in flight. The launch leaves the step loop together at
    the next cluster barrier, the call returns NBG_ERR_TIMEOUT with the state
    back at the chunk's start, and the next run on the same context is
    normal (against the oracle)."""
    sim = S.lj_liquid(1000, seed=21)
    desc, keep = nbg.system_descriptor(sim)
    u, v = S.state(sim)
    os.environ["NBG_TEST_CLUSTER_DROP"] = drop
    try:
        eng = nbg.Engine(desc, 0)
    finally:
        os.environ.pop("NBG_TEST_CLUSTER_DROP", None)
    assert eng.cluster_shape() is not None
    with pytest.raises(nbg.EngineError) as e:
        eng.run(u, v, 0.005, 20, 0, save_trajectory=False)
    assert e.value.status == -5  # NBG_ERR_TIMEOUT
    ug, vg, _, _, _ = eng.run(u, v, 0.005, 20, 0, save_trajectory=False)
    uo, vo = oracle.run(desc, u, v, 0.005, 20)
    assert np.abs(ug - uo).max() <= 1e-8 * np.abs(uo).max()
    eng.close()
