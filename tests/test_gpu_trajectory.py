"""Trajectory saving of nbg_run (run_simulation's save_everystep /
save_every, nbody_simulation_result.jl:480-487): the steps write the frames
into a device buffer (the graph step loop by a save kernel after each step,
the cluster step loop by its owner threads), copied out once per segment.
Saving must not change the dynamics, and frame j must be the state after
j * save_every steps, bit for bit."""
import os

import numpy as np
import pytest

import systems as S

nbg = S.nbg
pytestmark = pytest.mark.gpu


def _engine(kind):
    if kind == "lj_cluster":
        sim = S.lj_liquid(1000, seed=2)
        return sim, sim.engine(), 0.005
    if kind == "lj_graph":
        sim = S.lj_liquid(1000, seed=2)
        desc, keep = nbg.system_descriptor(sim)  # keep: the arrays desc points to, alive through creation
        os.environ["NBG_NO_CLUSTER"] = "1"
        try:
            return sim, nbg.Engine(desc, 0), 0.005
        finally:
            del os.environ["NBG_NO_CLUSTER"]
    if kind == "water":
        sim = S.water_box(216, seed=3, thermostat=nbg.BerendsenThermostat(300.0, 0.1))
        return sim, sim.engine(), 0.0005
    if kind == "gravity":
        sim = S.plummer(512)
        return sim, sim.engine(), 1e-3
    if kind == "langevin":
        sim = S.lj_liquid(500, seed=4, thermostat=nbg.LangevinThermostat(1.0, 1.0))
        return sim, sim.engine(), 0.005
    raise ValueError(kind)


@pytest.mark.parametrize("kind", ["lj_cluster", "lj_graph", "water", "gravity", "langevin"])
@pytest.mark.parametrize("every", [1, 3, 10])
def test_run_frames_match_unsaved_runs(gpu, kind, every):
    sim, eng, dt = _engine(kind)
    if kind == "lj_cluster":
        assert eng.cluster_shape() is not None
    if kind == "lj_graph":
        assert eng.cluster_shape() is None
    u0, v0 = S.state(sim)
    nsteps = 25
    u, v, tu, tv, _ = eng.run(u0, v0, dt, nsteps, every, step=0)
    nf = nsteps // every + 1 + (1 if nsteps % every else 0)
    assert len(tu) == nf and len(tv) == nf
    assert np.array_equal(tu[0], u0) and np.array_equal(tv[0], v0)
    assert np.array_equal(tu[-1], u) and np.array_equal(tv[-1], v)
    # saving changes nothing: the same run without frames
    u1, v1, _, _, _ = eng.run(u0, v0, dt, nsteps, 0, save_trajectory=False, step=0)
    assert np.array_equal(u1, u) and np.array_equal(v1, v)
    # frame j is the state after j * every steps
    for j in sorted({1, 2, nsteps // every}):
        uj, vj, _, _, _ = eng.run(u0, v0, dt, j * every, 0, save_trajectory=False, step=0)
        assert np.array_equal(tu[j], uj), (kind, every, j)
        assert np.array_equal(tv[j], vj), (kind, every, j)
    eng.close()


def test_run_frames_long_run(gpu):
    """2000 steps saved every step on the cluster path (one device segment of
    48 MB): a frame in the middle matches the end of a run without frames."""
    sim, eng, dt = _engine("lj_cluster")
    u0, v0 = S.state(sim)
    u, v, tu, tv, st = eng.run(u0, v0, dt, 2000, 1, step=0)
    assert len(tu) == 2001
    uj, _, _, _, _ = eng.run(u0, v0, dt, 1234, 0, save_trajectory=False, step=0)
    assert np.array_equal(tu[1234], uj)
    assert np.array_equal(tu[-1], u)
    eng.close()


@pytest.mark.parametrize("kind", ["lj_cluster", "lj_graph", "water", "gravity", "langevin"])
def test_run_frames_match_oracle_frames(gpu, oracle, kind):
    """save_every frames of nbg_run against the oracle's frames of the same
    run (the reference's saved solution, nbody_simulation_result.jl:480-487):
    positions within the trajectory tolerance of the parity tests (1e-8 of
    the coordinate scale after 20 steps; 1e-7 for Langevin), velocities
    within 1e-5 relative RMS (FP32 pair forces); the Langevin frames use the
    same Philox draws."""
    sim, eng, dt = _engine(kind)
    desc, keep = nbg.system_descriptor(sim)
    u0, v0 = S.state(sim)
    nsteps, every = 20, 5
    u, v, tu, tv, _ = eng.run(u0, v0, dt, nsteps, every, step=0)
    uo, vo, tuo, tvo = oracle.run(desc, u0, v0, dt, nsteps, every, trajectory=True)
    assert len(tu) == len(tuo) == nsteps // every + 1
    scale = max(np.abs(tuo).max(), 1.0)
    # Euler-Maruyama's FP32 Box-Muller normals add ~1e-7 relative noise errors
    tol = 1e-7 if kind == "langevin" else 1e-8
    for j in range(len(tu)):
        assert np.abs(tu[j] - tuo[j]).max() <= tol * scale, (kind, j, np.abs(tu[j] - tuo[j]).max())
        assert S.rel_rmse(tv[j], tvo[j]) <= 1e-5, (kind, j, S.rel_rmse(tv[j], tvo[j]))
    eng.close()
