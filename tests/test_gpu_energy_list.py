"""The O(N x neighbours) energy of list-path contexts against the O(N^2)
all-pairs sums (the reference's definitions) on the same positions."""
import numpy as np
import pytest

import __graft_entry__ as g
import systems

pytestmark = pytest.mark.gpu
nbg = g.load_package()


def _both(make):
    sim_l, u, v = make(0)
    sim_a, _, _ = make(nbg._abi.NBG_FLAG_ALL_PAIRS)
    return sim_l.engine(), sim_a.engine(), u, v


@pytest.mark.parametrize("eps_rf", [1.0, 78.5])
def test_water_list_energy_matches_all_pairs(gpu, eps_rf):
    def make(flags):
        sim, pos, vel, L = systems.spcfw_water_rf(1000, eps_rf=eps_rf)
        sim.flags = flags
        return sim, pos, vel
    el, ea, u, v = _both(make)
    el.set_state(u, v)
    el.advance(0.0005, 400)
    u, v = el.get_state()
    a, b = el.energy(u, v), ea.energy(u, v)
    for k in ("lennard_jones", "electrostatic", "bonds", "angles", "kinetic"):
        assert abs(a[k] - b[k]) <= 1e-10 * max(1.0, abs(b[k])), (k, a[k], b[k])


def test_lj_list_energy_matches_all_pairs(gpu):
    def make(flags):
        pos, vel, L = nbg.workloads.lj_argon_lattice(1000, rho=0.8, T=1.0, seed=2)
        bodies = [nbg.MassBody(pos[i], vel[i], 1.0) for i in range(len(pos))]
        sysm = nbg.PotentialNBodySystem(bodies, {"lennard_jones": nbg.LennardJonesParameters(1.0, 1.0, 2.5)})
        sim = nbg.NBodySimulation(sysm, (0.0, 1.0), nbg.CubicPeriodicBoundaryConditions(L), kb=1.0, skin=0.3,
                                  rebuild_every=10, flags=flags)
        return sim, pos, vel
    el, ea, u, v = _both(make)
    el.set_state(u, v)
    el.advance(0.005, 200)
    u, v = el.get_state()
    a, b = el.energy(u, v), ea.energy(u, v)
    assert abs(a["lennard_jones"] - b["lennard_jones"]) <= 1e-10 * abs(b["lennard_jones"])
