"""The persistent ensemble loop (k_ensemble.cu): a batch of replicas advanced
by one launch per chunk of steps, a CTA per replica with its positions in
shared memory and its Verlet lists rebuilt inside the launch.

Checked against the FP64 oracle (forces of every replica after the steps,
the pair classification of basic_potentials.jl:253-258 through them; BAOAB
steps with the same Philox draws), against the step-graph path of the same
batch, across launches (the lists carried over), and with trajectory frames
(nbody_simulation_result.jl:480-487)."""
import os

import numpy as np
import pytest

import systems as S

nbg = S.nbg
pytestmark = pytest.mark.gpu

FORCE_TOL = 1e-5


def _batch(sizes, langevin=True, seed=50):
    descs, keep, us, vs = [], [], [], []
    for r, n in enumerate(sizes):
        T = 0.8 + 0.2 * r
        pos, vel, L = nbg.workloads.lj_argon_lattice(n, seed=seed + r, jitter=0.05, T=T)
        th = nbg.LangevinThermostat(T, 1.0) if langevin else None
        d, k = nbg.lennard_jones_descriptor(np.ones(n), L, thermostat=th, seed=70 + r, skin=0.3,
                                            rebuild_every=10)
        if langevin:
            d.flags |= nbg._abi.NBG_FLAG_LANGEVIN_BAOAB
        descs.append(d)
        keep.append(k)
        us.append(pos)
        vs.append(vel)
    return descs, keep, np.concatenate(us), np.concatenate(vs)


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


SIZES = [150, 700, 2200, 4100, 8000]


@pytest.mark.parametrize("langevin", [True, False])
def test_loop_forces_match_oracle_and_graph_path(gpu, oracle, langevin):
    descs, keep, U, V = _batch(SIZES, langevin)
    eng = _engine(descs)
    assert eng.ensemble_form() is not None
    ref = _engine(descs, NBG_NO_ENSEMBLE_LOOP=1)
    assert ref.ensemble_form() is None
    dt = 0.005 if langevin else 0.004
    ug, vg, _, _, st = eng.run(U, V, dt, 40, 0, save_trajectory=False, step=0)
    ur, vr, _, _, _ = ref.run(U, V, dt, 40, 0, save_trajectory=False, step=0)
    assert np.all(np.isfinite(ug)) and np.all(np.isfinite(vg))
    # two FP32 force paths with different rounding, 40 chaotic steps apart by little
    assert np.abs(ug - ur).max() <= 1e-4, np.abs(ug - ur).max()
    a = eng.get_accel()
    off = 0
    for r, n in enumerate(SIZES):
        ao, _ = oracle.accel(descs[r], vg[off:off + n].copy(), ug[off:off + n])
        assert S.rel_rmse(a[off:off + n], ao) <= FORCE_TOL, (r, S.rel_rmse(a[off:off + n], ao))
        off += n
    eng.close()
    ref.close()


def test_loop_baoab_steps_match_oracle(gpu, oracle):
    """Three BAOAB steps of every replica against the oracle's (same Philox
    draws: FP32 Box-Muller on the GPU)."""
    descs, keep, U, V = _batch(SIZES, True)
    eng = _engine(descs)
    ug, vg, _, _, _ = eng.run(U, V, 0.005, 3, 0, save_trajectory=False, step=0)
    off = 0
    for r, n in enumerate(SIZES):
        uo, vo = oracle.run(descs[r], U[off:off + n], V[off:off + n], 0.005, 3)
        assert np.abs(ug[off:off + n] - uo).max() <= 1e-6 * descs[r].box[0]
        assert np.abs(vg[off:off + n] - vo).max() <= 1e-5 * np.abs(vo).max()
        off += n
    eng.close()


def test_loop_launches_continue_bit_for_bit(gpu):
    """Two 30-step runs (the second continuing the counter, the lists carried
    over to its launch) equal one 60-step run bit for bit; a run split by
    nbg_advance calls too."""
    descs, keep, U, V = _batch(SIZES, True)
    eng = _engine(descs)
    u60, v60, _, _, _ = eng.run(U, V, 0.005, 60, 0, save_trajectory=False, step=0)
    eng.set_step(0)
    eng.set_state(U, V)
    eng.advance(0.005, 30)
    eng.advance(0.005, 30)
    u2, v2 = eng.get_state()
    assert np.array_equal(u2, u60) and np.array_equal(v2, v60)
    eng.close()


@pytest.mark.parametrize("every", [1, 7])
def test_loop_frames(gpu, every):
    descs, keep, U, V = _batch(SIZES, True)
    eng = _engine(descs)
    u, v, tu, tv, _ = eng.run(U, V, 0.005, 21, every, step=0)
    u1, v1, _, _, _ = eng.run(U, V, 0.005, 21, 0, save_trajectory=False, step=0)
    assert np.array_equal(u1, u) and np.array_equal(v1, v)
    for j in sorted({1, 21 // every}):
        uj, vj, _, _, _ = eng.run(U, V, 0.005, j * every, 0, save_trajectory=False, step=0)
        assert np.array_equal(tu[j], uj) and np.array_equal(tv[j], vj)
    eng.close()


def test_loop_pair_sets_after_steps(gpu, oracle):
    """After steps on the loop, the pair sets of the largest and smallest
    replica (the same classification code) equal the reference's."""
    descs, keep, U, V = _batch(SIZES, True)
    eng = _engine(descs)
    ug, vg, _, _, _ = eng.run(U, V, 0.005, 25, 0, save_trajectory=False, step=0)
    gp = eng.pair_list(ug, nbg._abi.NBG_POT_LJ)
    starts = np.concatenate([[0], np.cumsum(SIZES)])
    for r in (0, len(SIZES) - 1):
        lo, hi = starts[r], starts[r + 1]
        a0, b0 = np.searchsorted(gp[:, 0], [lo, hi])
        ref = oracle.pair_list(descs[r], ug[lo:hi], nbg._abi.NBG_POT_LJ)
        assert np.array_equal(gp[a0:b0] - lo, ref)
    eng.close()


def test_loop_tuner_keeps_results(gpu, oracle):
    """The tuner times every form of the loop on a copy of the state and
    keeps the fastest; the state and the step counter are unchanged, and the
    chosen form's forces still match the oracle."""
    descs, keep, U, V = _batch(SIZES, True)
    eng = _engine(descs)
    eng.set_state(U, V)
    eng.set_step(5)
    form, ms = eng.ensemble_tune(3)
    assert len(ms) == 13 and np.all(np.isfinite(ms)) and np.all(ms > 0)
    assert (form is None) == (int(np.argmin(ms)) == 12)
    assert eng.step == 5
    u, v = eng.get_state()
    assert np.array_equal(u, U) and np.array_equal(v, V)
    assert eng.ensemble_form() == form
    ug, vg, _, _, _ = eng.run(U, V, 0.005, 20, 0, save_trajectory=False, step=0)
    a = eng.get_accel()
    off = 0
    for r, n in enumerate(SIZES):
        ao, _ = oracle.accel(descs[r], vg[off:off + n].copy(), ug[off:off + n])
        assert S.rel_rmse(a[off:off + n], ao) <= FORCE_TOL
        off += n
    eng.close()
