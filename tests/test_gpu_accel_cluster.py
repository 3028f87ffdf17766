"""nbg_accel of a small system (up to 2048 atoms, one replica, cubic box, no
thermostat) as one cluster launch: the right-hand side soode_system!
(nbody_to_ode.jl:471-489) with the LJ pair set of basic_potentials.jl:253-258
under the minimum image (boundary_conditions.jl:138-165).

The launch reads u and writes dv in place when they are page-locked host
buffers, else through the library's pinned staging: both give the same
numbers bit for bit. Its lists are its own, kept between calls while no atom
moved more than skin/2 from their build; the results match the oracle and the
graph path (NBG_NO_CLUSTER) on a walk of small and large displacements, and
the resident state is not touched.

Also the queued (nbg_advance) cluster chunk whose status comes back through
the mapped status word: a timeout in a launch on a state whose acceleration
is known (the launch writes its own backup) restores that launch's start."""
import os

import numpy as np
import pytest

import systems as S

nbg = S.nbg
pytestmark = pytest.mark.gpu

FORCE_TOL = 1e-5


def _engine(desc, **env):
    old = {k: os.environ.get(k) for k in env}
    os.environ.update({k: str(v) for k, v in env.items()})
    try:
        return nbg.Engine(desc, 0)
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


def _pinned(a):
    import torch
    t = torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).pin_memory()
    return t, t.numpy()


@pytest.mark.parametrize("n", [512, 1000, 1728])
def test_accel_cluster_pinned_and_pageable_match_oracle(gpu, oracle, n):
    sim = S.lj_liquid(n, seed=31, jitter=0.05)
    desc, keep = nbg.system_descriptor(sim)
    u, v = S.state(sim)
    eng = _engine(desc)
    assert eng.cluster_shape() is not None
    ref = _engine(desc, NBG_NO_CLUSTER=1)
    assert ref.cluster_shape() is None
    a_page = eng.accel(v.copy(), u)
    ut, up = _pinned(u)
    at, ap = _pinned(np.zeros_like(u))
    eng.accel(v.copy(), up, out=ap)
    assert np.array_equal(a_page, ap)
    a_ref = ref.accel(v.copy(), u)
    # two FP32 force paths (split positions here, fixed point there)
    assert S.rel_rmse(a_page, a_ref) <= 5e-6, S.rel_rmse(a_page, a_ref)
    ao, _ = oracle.accel(desc, v.copy(), u)
    assert S.rel_rmse(a_page, ao) <= FORCE_TOL, S.rel_rmse(a_page, ao)
    eng.close()
    ref.close()


def test_accel_cluster_lists_across_calls(gpu, oracle):
    """A walk of small displacements (lists kept), then a jump (rebuilt),
    then back: every call against the oracle and the graph path."""
    sim = S.lj_liquid(1000, seed=32, jitter=0.05)
    desc, keep = nbg.system_descriptor(sim)
    u0, v = S.state(sim)
    eng = _engine(desc)
    ref = _engine(desc, NBG_NO_CLUSTER=1)
    rng = np.random.default_rng(5)
    ut, up = _pinned(u0)
    at, ap = _pinned(np.zeros_like(u0))
    u = u0.copy()
    for k in range(14):
        if k == 9:
            u = u + 0.5 * rng.standard_normal(u.shape)  # beyond skin / 2: the lists are rebuilt
        elif k == 12:
            u = u0.copy()
        else:
            u = u + 0.02 * rng.standard_normal(u.shape)
        up[:] = u
        eng.accel(v.copy(), up, out=ap)
        a_ref = ref.accel(v.copy(), u)
        assert S.rel_rmse(ap, a_ref) <= 5e-6, (k, S.rel_rmse(ap, a_ref))
        if k % 3 == 0 or k >= 9:
            ao, _ = oracle.accel(desc, v.copy(), u)
            assert S.rel_rmse(ap, ao) <= FORCE_TOL, (k, S.rel_rmse(ap, ao))
    eng.close()
    ref.close()


def test_accel_cluster_leaves_resident_state(gpu):
    """nbg_accel calls between queued steps do not change the steps."""
    sim = S.lj_liquid(1000, seed=33, jitter=0.05)
    desc, keep = nbg.system_descriptor(sim)
    u, v = S.state(sim)
    eng = _engine(desc)
    u20, v20, _, _, _ = eng.run(u, v, 0.005, 20, 0, save_trajectory=False, step=0)
    eng.set_state(u, v)
    eng.advance(0.005, 10)
    rng = np.random.default_rng(6)
    eng.accel(v.copy(), u + 0.3 * rng.standard_normal(u.shape))
    eng.advance(0.005, 10)
    eng.sync()
    u2, v2 = eng.get_state()
    assert np.array_equal(u2, u20) and np.array_equal(v2, v20)
    eng.close()


def test_queued_cluster_chunk_timeout_restores_its_start(gpu, oracle):
    """NBG_TEST_CLUSTER_DROP "3:1": the second cluster launch drops the
    position copies of its step 3. That launch runs on a state whose
    acceleration is known, so it writes its own backup and reports to the
    mapped status word; nbg_sync returns NBG_ERR_TIMEOUT with the state and
    the step counter back at the launch's start, and the context goes on
    normally."""
    sim = S.lj_liquid(1000, seed=21)
    desc, keep = nbg.system_descriptor(sim)
    u, v = S.state(sim)
    eng = _engine(desc, NBG_TEST_CLUSTER_DROP="3:1")
    assert eng.cluster_shape() is not None
    eng.set_state(u, v)
    eng.set_step(0)
    eng.advance(0.005, 10)
    eng.sync()
    u10, v10 = eng.get_state()
    eng.advance(0.005, 10)
    with pytest.raises(nbg.EngineError) as e:
        eng.sync()
    assert e.value.status == -5  # NBG_ERR_TIMEOUT
    assert eng.step == 10
    u1, v1 = eng.get_state()
    assert np.array_equal(u1, u10) and np.array_equal(v1, v10)
    eng.advance(0.005, 10)
    eng.sync()
    ug, vg = eng.get_state()
    uo, vo = oracle.run(desc, u, v, 0.005, 20)
    assert np.abs(ug - uo).max() <= 1e-8 * np.abs(uo).max()
    eng.close()


def test_cluster_launch_floor(gpu):
    """The launch floor of the cluster loop's shape (an empty kernel with the
    same CTAs, threads, shared memory and cluster): positive and finite (the
    two timings are not ordered: both are averages on a shared device); off
    the cluster path it is NBG_ERR_UNSUPPORTED."""
    sim = S.lj_liquid(1000, seed=34)
    desc, keep = nbg.system_descriptor(sim)
    eng = _engine(desc)
    single, b2b = eng.cluster_launch_floor()
    assert 0.0 < b2b < 1000.0 and 0.0 < single < 1000.0
    ref = _engine(desc, NBG_NO_CLUSTER=1)
    assert ref.cluster_launch_floor() is None
    eng.close()
    ref.close()
