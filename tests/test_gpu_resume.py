"""Resumable noise: the context's step counter keys the Philox draws of the
Andersen collisions (nbody_simulation_result.jl:504-540) and of the Langevin
SDE (nbody_to_ode.jl:567-680). It keeps running across nbg_run calls, so
every run draws fresh noise as each run_simulation call of the reference
does, and nbg_get_step / nbg_set_step make a checkpoint (state + counter)
resumable bit for bit.

Also the water Langevin SDE against the oracle (nbody_to_ode.jl:600-680:
the O rows lose gamma v / m_O inside the O loop, the H rows are reset by the
H loop, every row loses gamma v at the end, sigma = sqrt(2 gamma kb T) / m
per atom) and the reference's water thermostating test
(test/water_test.jl:136-153)."""
import numpy as np
import pytest

import systems as S

nbg = S.nbg
pytestmark = pytest.mark.gpu


def _noisy(kind):
    if kind == "em":
        return S.lj_liquid(1000, seed=6, thermostat=nbg.LangevinThermostat(1.0, 1.0)), 0.002
    if kind == "baoab":
        return S.lj_liquid(1000, seed=6, thermostat=nbg.LangevinThermostat(1.0, 1.0),
                           flags=nbg._abi.NBG_FLAG_LANGEVIN_BAOAB), 0.005
    return S.lj_liquid(1000, seed=7, thermostat=nbg.AndersenThermostat(1.0, 5.0)), 0.005


@pytest.mark.parametrize("kind", ["em", "baoab", "andersen"])
def test_two_segments_equal_one_run(gpu, kind):
    """Two 50-step nbg_run segments (the second continuing the counter) equal
    one 100-step run bit for bit: the resume point 50 is a multiple of
    rebuild_every (10), where the uninterrupted run rebuilds its lists too."""
    sim, dt = _noisy(kind)
    desc, keep = nbg.system_descriptor(sim)
    u0, v0 = S.state(sim)
    eng = nbg.Engine(desc, 0)
    u100, v100, _, _, _ = eng.run(u0, v0, dt, 100, 0, save_trajectory=False, step=0)
    assert eng.step == 100
    u50, v50, _, _, _ = eng.run(u0, v0, dt, 50, 0, save_trajectory=False, step=0)
    assert eng.step == 50
    u2, v2, _, _, _ = eng.run(u50, v50, dt, 50, 0, save_trajectory=False)
    assert eng.step == 100
    assert np.array_equal(u2, u100) and np.array_equal(v2, v100)
    # a checkpoint (state and counter) restored into a fresh context
    other = nbg.Engine(desc, 0)
    other.set_step(50)
    u3, v3, _, _, _ = other.run(u50, v50, dt, 50, 0, save_trajectory=False)
    assert np.array_equal(u3, u100) and np.array_equal(v3, v100)
    other.close()
    eng.close()


@pytest.mark.parametrize("kind", ["em", "andersen"])
def test_runs_draw_fresh_noise(gpu, kind):
    """Two runs from the same state continue the counter: different noise,
    as two run_simulation calls of the reference draw different numbers; the
    counter set back to 0 replays the first run."""
    sim, dt = _noisy(kind)
    desc, keep = nbg.system_descriptor(sim)
    u0, v0 = S.state(sim)
    eng = nbg.Engine(desc, 0)
    ua, va, _, _, _ = eng.run(u0, v0, dt, 10, 0, save_trajectory=False, step=0)
    ub, vb, _, _, _ = eng.run(u0, v0, dt, 10, 0, save_trajectory=False)
    assert not np.array_equal(va, vb)
    uc, vc, _, _, _ = eng.run(u0, v0, dt, 10, 0, save_trajectory=False, step=0)
    assert np.array_equal(ua, uc) and np.array_equal(va, vc)
    with pytest.raises(nbg.EngineError):
        eng.set_step(-1)
    eng.close()


def test_frames_of_a_continued_run(gpu):
    """The frame slots count from the run's first step, whatever the counter
    is: frames of a run started at step 37 match separate runs from there."""
    sim, dt = _noisy("em")
    desc, keep = nbg.system_descriptor(sim)
    u0, v0 = S.state(sim)
    eng = nbg.Engine(desc, 0)
    u, v, tu, tv, _ = eng.run(u0, v0, dt, 12, 4, step=37)
    assert len(tu) == 4 and np.array_equal(tu[0], u0) and np.array_equal(tu[-1], u)
    for j in (1, 2):
        uj, vj, _, _, _ = eng.run(u0, v0, dt, 4 * j, 0, save_trajectory=False, step=37)
        assert np.array_equal(tu[j], uj) and np.array_equal(tv[j], vj)
    eng.close()


def _ref_water_langevin(T0=275.0, gamma=100.0, n_mol=216, seed=5):
    """test/water_test.jl:5-31,136-153: the reference's SPC/Fw parameters,
    bodies on the cell nodes, Langevin thermostat (T0, gamma)."""
    w = S.WATER
    L, lj, el, spc, mH2O = S.water_params(n_mol)
    v_dev = (S.KB_KJ * w["T"] / mH2O) ** 0.5
    bodies = nbg.generate_bodies_in_cell_nodes(n_mol, mH2O, v_dev, L, rng=np.random.default_rng(seed))
    water = nbg.WaterSPCFw(bodies, w["mH"], w["mO"], w["qH"], w["qO"], lj, el, spc)
    # t2 = 200 tau' with tau' = 0.5e-4 ps, stepped at dt = tau = 0.5e-3 ps: 20 steps
    return nbg.NBodySimulation(water, (0.0, 200 * 0.5e-4), nbg.CubicPeriodicBoundaryConditions(L),
                               nbg.LangevinThermostat(T0, gamma), S.KB_KJ), w["tau"]


def test_water_langevin_em_matches_oracle(gpu, oracle):
    """Three Euler-Maruyama steps of the water SDE with the same Philox draws
    (FP32 Box-Muller and FP32 pair forces on the GPU, FP64 in the oracle)."""
    sim, tau = _ref_water_langevin()
    desc, keep = nbg.system_descriptor(sim)
    u, v = S.state(sim)
    ug, vg, _, _, _ = nbg.Engine(desc, 0).run(u, v, tau, 3, 0, save_trajectory=False, step=0)
    uo, vo = oracle.run(desc, u, v, tau, 3)
    assert S.rel_rmse(ug - u, uo - u) <= 1e-5, S.rel_rmse(ug - u, uo - u)
    assert S.rel_rmse(vg, vo) <= 1e-5, S.rel_rmse(vg, vo)


def test_water_langevin_thermostating(gpu):
    """test/water_test.jl:136-153: 216 molecules, LangevinThermostat(275, 100),
    EM at dt = tau = 0.5 fs up to t2 = 10 fs (20 steps): |T(t2) - T0| / T0
    within 1."""
    sim, tau = _ref_water_langevin()
    result = nbg.run_simulation(sim, nbg.EM(), dt=tau)
    T2 = nbg.temperature(result, sim.tspan[1])
    assert np.isfinite(T2) and abs(T2 - 275.0) / 275.0 <= 1.0
