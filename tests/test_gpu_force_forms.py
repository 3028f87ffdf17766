"""The Verlet-list force kernel's forms on the same inputs: the fixed-point
kernel with TMA-staged lists (every lanes-per-atom width) against the
split-position kernels and the FP64 oracle (basic_potentials.jl:240-304),
on LJ, LJ + electrostatics, water and an uneven batch."""
import os

import numpy as np
import pytest

import systems as S

nbg = S.nbg
pytestmark = pytest.mark.gpu

FORCE_TOL = 1e-5


def _engine(descs, **env):
    old = {k: os.environ.get(k) for k in env}
    os.environ.update({k: str(v) for k, v in env.items()})
    try:
        return nbg.Engine(descs, 0)
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


def _forces(eng, u, v):
    eng.set_state(u, v)
    eng.compute_forces()
    return eng.get_accel()


def _systems():
    out = {}
    sim = S.lj_liquid(1000, seed=11, jitter=0.1)
    out["lj"] = sim
    pos, vel, L = nbg.workloads.lj_argon_lattice(1000, seed=9, jitter=0.1)
    rng = np.random.default_rng(9)
    bodies = [nbg.ChargedParticle(pos[i], vel[i], 1.0, rng.choice([-0.5, 0.5])) for i in range(len(pos))]
    system = nbg.PotentialNBodySystem(bodies, {"lennard_jones": nbg.LennardJonesParameters(1.0, 1.0, 2.5),
                                               "electrostatic": nbg.ElectrostaticParameters(1.0, 3.0)})
    out["ljel"] = nbg.NBodySimulation(system, (0.0, 1.0), nbg.CubicPeriodicBoundaryConditions(L), kb=1.0, skin=0.3)
    out["water"] = S.water_box(1000, seed=6)
    out["water_rf"] = S.water_box(1000, seed=7, eps_rf=78.5)
    return out


@pytest.mark.parametrize("name", ["lj", "ljel", "water", "water_rf"])
@pytest.mark.parametrize("lanes,staging", [(4, "warp"), (8, "warp"), (16, "warp"), (4, "block"), (8, "block"),
                                           (16, "block"), (32, "block")])
def test_fixed_point_kernel_matches_oracle_and_split_form(gpu, oracle, name, lanes, staging):
    """Both stagings of the lists (per warp: a ring of 32-entry boxes; per
    block: whole tiles, double-buffered) at every width."""
    sim = _systems()[name]
    desc, keep = nbg.system_descriptor(sim)
    u, v = S.state(sim)
    extra = {"NBG_FX_BLOCK": 1} if staging == "block" and lanes < 32 else {}
    eng = _engine(desc, NBG_LIST_LPA=lanes, NBG_NO_CLUSTER=1, **extra)
    # water's ~580-entry list rows for 64 atoms of 4 lanes overflow the two
    # per-block shared-memory stages: that form stays on the split-position kernel
    assert eng.force_form() == (lanes, not (name.startswith("water") and lanes == 4 and staging == "block"))
    ref = _engine(desc, NBG_LIST_LPA=lanes, NBG_NO_CLUSTER=1, NBG_NO_FX=1)
    assert ref.force_form() == (lanes, False)
    a_fx = _forces(eng, u, v)
    a_split = _forces(ref, u, v)
    assert S.rel_rmse(a_fx, a_split) <= 2e-6
    if desc.el_eps_rf == 1.0:  # the oracle restates the reference's truncated Coulomb only
        a_or, _ = oracle.accel(desc, v.copy(), u)
        assert S.rel_rmse(a_fx, a_or) <= FORCE_TOL, S.rel_rmse(a_fx, a_or)
    # the pair sets the two forms count are the reference's, bit for bit
    for which in (nbg._abi.NBG_POT_LJ, nbg._abi.NBG_POT_EL):
        if not (desc.potentials & which or desc.kind == nbg._abi.NBG_SYSTEM_WATER):
            continue
        po = oracle.pair_list(desc, u, which)
        assert np.array_equal(eng.pair_list(u, which), po)
    eng.close()
    ref.close()


def test_fixed_point_batch_and_steps(gpu, oracle):
    """An uneven batch (one-cell and many-cell replicas): forces after 30
    BAOAB steps through the fixed-point kernel against each replica's
    oracle, and the run against the split-form run to rounding."""
    sizes = [200, 1200, 3000]
    descs, keep, us, vs = [], [], [], []
    for r, n in enumerate(sizes):
        pos, vel, L = nbg.workloads.lj_argon_lattice(n, seed=30 + r, jitter=0.05, T=1.2)
        d, k = nbg.lennard_jones_descriptor(np.ones(n), L, thermostat=nbg.LangevinThermostat(1.2, 1.0),
                                            seed=40 + r, skin=0.3, rebuild_every=10)
        d.flags |= nbg._abi.NBG_FLAG_LANGEVIN_BAOAB
        descs.append(d)
        keep.append(k)
        us.append(pos)
        vs.append(vel)
    U, V = np.concatenate(us), np.concatenate(vs)
    eng = _engine(descs, NBG_LIST_LPA=4)
    ref = _engine(descs, NBG_LIST_LPA=4, NBG_NO_FX=1)
    assert eng.force_form() == (4, True) and ref.force_form() == (4, False)
    ug, vg, _, _, _ = eng.run(U, V, 0.005, 30, 0, save_trajectory=False, step=0)
    ur, vr, _, _, _ = ref.run(U, V, 0.005, 30, 0, save_trajectory=False, step=0)
    # two FP32 kernels with different rounding: 30 chaotic steps apart by little
    assert np.abs(ug - ur).max() <= 5e-5
    a = eng.get_accel()
    off = 0
    for r, n in enumerate(sizes):
        ao, _ = oracle.accel(descs[r], vg[off:off + n].copy(), ug[off:off + n])
        assert S.rel_rmse(a[off:off + n], ao) <= FORCE_TOL
        off += n
    eng.close()
    ref.close()
