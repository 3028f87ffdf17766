"""CPU checks of the FP64 restatement of the learned short-range model
(oracle/learned.py): its forces are the negative gradients of its energies,
and the training gradient is the gradient of the batch loss."""
import math

import numpy as np
import pytest

import __graft_entry__ as g
import systems

LO = g.load_learned_oracle()


@pytest.fixture(scope="module")
def small_box():
    pos, vel, L = systems.nbg.workloads.spcfw_water_box(64, seed=5)
    rng = np.random.default_rng(3)
    pos = pos + rng.normal(scale=0.004, size=pos.shape)
    q = np.tile([-0.82, 0.41, 0.41], 64)
    return pos, L, q


def _params(seed, D, E):
    rng = np.random.default_rng(seed)
    th = np.zeros(LO.n_params())
    th[:64 * 128] = 0.3 * rng.standard_normal(64 * 128) / 8
    o = 64 * 128 + 128
    th[o:o + 128 * 128] = rng.standard_normal(128 * 128) / math.sqrt(128)
    o2 = o + 128 * 128 + 128
    th[o2:o2 + 128] = rng.standard_normal(128) / math.sqrt(128)
    n = 24961
    th[n:n + 64] = D.mean(axis=0)
    th[n + 64:n + 128] = D.std(axis=0) + 1e-3
    th[n + 128], th[n + 129] = E.mean(), E.std()
    return th


def test_learned_forces_are_negative_energy_gradient(small_box):
    u, L, q = small_box
    D = np.array([LO.descriptor(u, L, i)[0] for i in range(len(u))])
    E, _ = LO.short_range_labels(u, L, q, 0.650299, 0.3165492, 138.935458)
    th = [_params(1, D, E), _params(2, D, E)]
    _, F = LO.forces(u, L, th)
    h = 1e-6
    for i, k in ((0, 0), (1, 2), (5, 1), (100, 0)):
        up, um = u.copy(), u.copy()
        up[i, k] += h
        um[i, k] -= h
        fd = -(LO.forces(up, L, th)[0] - LO.forces(um, L, th)[0]) / (2 * h)
        assert abs(fd - F[i, k]) <= 1e-6 * max(1.0, abs(F[i, k])), (i, k, fd, F[i, k])


def test_short_range_labels_forces_are_negative_gradient(small_box):
    u, L, q = small_box
    E, F = LO.short_range_labels(u, L, q, 0.650299, 0.3165492, 138.935458)
    h = 1e-6
    for i, k in ((0, 0), (2, 1), (33, 2)):
        up, um = u.copy(), u.copy()
        up[i, k] += h
        um[i, k] -= h
        Ep = LO.short_range_labels(up, L, q, 0.650299, 0.3165492, 138.935458)[0].sum()
        Em = LO.short_range_labels(um, L, q, 0.650299, 0.3165492, 138.935458)[0].sum()
        fd = -(Ep - Em) / (2 * h)
        assert abs(fd - F[i, k]) <= 1e-6 * max(1.0, abs(F[i, k])), (i, k, fd, F[i, k])


def test_training_gradient_is_loss_gradient():
    rng = np.random.default_rng(7)
    D = rng.standard_normal((200, 64))
    th = _params(4, D, rng.standard_normal(200))
    X = rng.standard_normal((16, 64))
    y = rng.standard_normal(16)
    loss, grad = LO.train_gradients(th, X, y)
    h = 1e-6
    for p in (0, 5000, 64 * 128 + 3, 64 * 128 + 128 + 777, 24961 - 1, 24961 - 50):
        tp, tm = th.copy(), th.copy()
        tp[p] += h
        tm[p] -= h
        fd = (LO.train_gradients(tp, X, y)[0] - LO.train_gradients(tm, X, y)[0]) / (2 * h)
        assert abs(fd - grad[p]) <= 1e-6 * max(1.0, abs(grad[p])), (p, fd, grad[p])


def test_sampled_forces_and_labels_equal_full_rows(small_box):
    """forces_on / labels_on (the sampled forms the full-size GPU checks use)
    give the rows of forces / short_range_labels of the whole box."""
    u, L, q = small_box
    D = np.array([LO.descriptor(u, L, i)[0] for i in range(len(u))])
    E, F = LO.short_range_labels(u, L, q, 0.650299, 0.3165492, 138.935458)
    th = [_params(7, D, E), _params(8, D, E)]
    _, Ff = LO.forces(u, L, th)
    idx = np.array([0, 1, 2, 50, 97, 191])
    Fs = LO.forces_on(u, L, th, idx)
    assert np.abs(Fs - Ff[idx]).max() <= 1e-10 * np.abs(Ff).max()
    Es, Fl = LO.labels_on(u, L, q, 0.650299, 0.3165492, 138.935458, idx)
    assert np.array_equal(Es, E[idx]) and np.array_equal(Fl, F[idx])


def test_oracle_partial_accel_rows_of_water(small_box):
    """oracle_partial_accel over whole molecules (with their angle terms)
    equals the rows of the full right-hand side."""
    import systems as S
    sim = S.water_box(64, seed=5)
    desc, keep = S.nbg.system_descriptor(sim)
    u, v = S.state(sim)
    oracle = g.load_oracle()
    a, _ = oracle.accel(desc, v.copy(), u)
    for i0, i1 in ((0, 30), (99, 192)):
        p = oracle.partial_accel(desc, u, i0, i1)
        assert np.abs(p - a[i0:i1]).max() <= 1e-12 * np.abs(a).max()
