"""Parity at the benchmark configurations' full sizes: the CUDA path against
the FP64 oracle on the very systems the throughput numbers are quoted on.

- All-pairs gravity, 65,536-body Plummer sphere (basic_potentials.jl:306-331):
  accelerations of 1,024 bodies in four blocks against the oracle's per-body
  loops, compensated and plain FP32, through the drop-in nbg_accel and after
  20 resident velocity-Verlet steps (the Morton sort schedule in between).
- SPC/Fw water, 4,096 molecules with the benchmark's parameters and the
  reference's truncated Coulomb (eps_rf = 1): both pair sets in full against
  the reference's r^2 < R^2 (basic_potentials.jl:253-258, 288-292 with the
  minimum image of boundary_conditions.jl:138-165), and the accelerations of
  1,200 atoms (whole molecules, bonds and angles included), at the start and
  after 20 Berendsen steps.
- The uneven 256-replica Langevin ensemble (1.08 M atoms): after 20 BAOAB
  steps (rebuilds have happened), the resident accelerations of sampled atoms
  of 16 replicas against the oracle, and the pair sets of the smallest, the
  median and the largest replica in full, all through the one batch context.
- The learned model on 98,304 atoms: descriptors and short-range labels of
  256 sampled atoms, learned BF16 forces of 48 sampled atoms (from their
  local neighbourhoods in oracle/learned.py)."""
import math

import numpy as np
import pytest

import __graft_entry__ as g
import bench
import systems as S

nbg = S.nbg
pytestmark = pytest.mark.gpu

FORCE_TOL = 1e-5  # relative RMS force error against the FP64 oracle


def _rows(a, blocks):
    return np.concatenate([a[i0:i1] for i0, i1 in blocks])


def _oracle_rows(oracle, desc, u, blocks):
    return np.concatenate([oracle.partial_accel(desc, u, i0, i1) for i0, i1 in blocks])


@pytest.mark.parametrize("plain", [False, True])
def test_gravity_plummer_65536(gpu, oracle, plain):
    wl = bench.Workload(nbg, "gravity")
    desc = wl.descs[0]
    if plain:
        desc.flags |= nbg._abi.NBG_FLAG_GRAV_PLAIN
    n = int(desc.n)
    assert n == 65536
    blocks = [(0, 256), (20000, 20256), (41000, 41256), (n - 256, n)]
    eng = nbg.Engine(desc, 0)
    u, v = wl.u0, wl.v0
    a = eng.accel(v.copy(), u)
    err = S.rel_rmse(_rows(a, blocks), _oracle_rows(oracle, desc, u, blocks))
    # compensated: differences accurate to 2^-24 |r_ij|; plain FP32 positions
    assert err <= (FORCE_TOL if plain else 1e-6), err
    # resident steps: accelerations of the state after 20 steps (the Morton
    # sort ran on evaluations 0, 8 and 16)
    eng.set_state(u, v)
    eng.advance(1e-3, 20)
    u20, _ = eng.get_state()
    eng.compute_forces()
    a20 = eng.get_accel()
    err20 = S.rel_rmse(_rows(a20, blocks), _oracle_rows(oracle, desc, u20, blocks))
    assert err20 <= (FORCE_TOL if plain else 1e-6), err20
    eng.close()


def _pair_sets_equal(eng, oracle, desc, u, which):
    gp = eng.pair_list(u, which)
    op = oracle.pair_list(desc, u, which)
    assert gp.shape == op.shape, (gp.shape, op.shape)
    assert np.array_equal(gp, op)
    return len(op)


def test_water_4096_pair_sets_and_forces(gpu, oracle):
    wl = bench.Workload(nbg, "water")
    desc = wl.descs[0]
    assert int(desc.n) == 12288 and desc.el_eps_rf == 1.0
    eng = nbg.Engine(desc, 0)
    u, v = wl.u0, wl.v0
    blocks = [(0, 300), (4500, 4800), (9000, 9300), (11988, 12288)]
    for state in range(2):
        n_lj = _pair_sets_equal(eng, oracle, desc, u, nbg._abi.NBG_POT_LJ)
        n_el = _pair_sets_equal(eng, oracle, desc, u, nbg._abi.NBG_POT_EL)
        assert n_lj > 4096 * 80 and n_el > 12288 * 250  # ~92 O and ~295 EL partners within 0.9 nm
        eng.set_state(u, v)
        eng.compute_forces()
        a = eng.get_accel()
        err = S.rel_rmse(_rows(a, blocks), _oracle_rows(oracle, desc, u, blocks))
        assert err <= FORCE_TOL, (state, err)
        if state == 0:
            u, v, _, _, _ = eng.run(u, v, 0.0005, 20, 0, save_trajectory=False)
    eng.close()


def test_ensemble_256_replicas(gpu, oracle):
    wl = bench.Workload(nbg, "ensemble")
    sizes = wl.sizes
    assert len(sizes) == 256
    starts = np.concatenate([[0], np.cumsum(sizes)])
    eng = nbg.Engine(wl.descs, 0)
    u, v, _, _, st = eng.run(wl.u0, wl.v0, 0.005, 20, 0, save_trajectory=False)
    assert st.list_builds > 256  # replicas rebuilt on displacement within the 20 steps
    a = eng.get_accel()
    order = np.argsort(sizes)
    picks = sorted(set(order[np.linspace(0, 255, 16).astype(int)].tolist()))
    got, want = [], []
    for r in picks:
        n = sizes[r]
        ur = u[starts[r]:starts[r + 1]]
        for i0 in (0, n // 2, n - 64):
            got.append(a[starts[r] + i0:starts[r] + i0 + 64])
            want.append(oracle.partial_accel(wl.descs[r], ur, i0, i0 + 64))
    err = S.rel_rmse(np.concatenate(got), np.concatenate(want))
    assert err <= FORCE_TOL, err
    # pair sets of the smallest, median and largest replica, from the batch
    gp = eng.pair_list(u, nbg._abi.NBG_POT_LJ)
    for r in (order[0], order[128], order[-1]):
        lo, hi = starts[r], starts[r + 1]
        a0, b0 = np.searchsorted(gp[:, 0], [lo, hi])
        mine = gp[a0:b0] - lo
        ref = oracle.pair_list(wl.descs[r], u[lo:hi], nbg._abi.NBG_POT_LJ)
        assert mine.shape == ref.shape and np.array_equal(mine, ref), r
        assert np.all((gp[a0:b0, 1] >= lo) & (gp[a0:b0, 1] < hi))  # no pair crosses replicas
    eng.close()


def _random_params(seed, D, E):
    rng = np.random.default_rng(seed)
    th = np.zeros(nbg._abi.NBG_ML_NPARAM)
    th[:64 * 128] = 0.1 * rng.standard_normal(64 * 128) / 8
    o = 64 * 128 + 128
    th[o:o + 128 * 128] = rng.standard_normal(128 * 128) / math.sqrt(128)
    o2 = o + 128 * 128 + 128
    th[o2:o2 + 128] = rng.standard_normal(128) / math.sqrt(128)
    th[o2 + 128] = 0.3
    n = nbg._abi.NBG_ML_NTRAIN
    th[n:n + 64] = D.mean(axis=0)
    th[n + 64:n + 128] = D.std(axis=0) + 1e-3
    th[n + 128], th[n + 129] = E.mean(), E.std()
    return th.astype(np.float32)


def test_learned_model_98304(gpu):
    LO = g.load_learned_oracle()
    sim, pos, vel = bench.mts_sim(nbg, 32768)
    L = sim.boundary_conditions.L
    eng = sim.engine()
    eng.set_state(pos, vel)
    eng.advance(0.0005, 100)  # off the lattice
    u, _ = eng.get_state()
    n = len(u)
    assert n == 98304
    eng.ml_enable()
    q = np.tile([-0.82, 0.41, 0.41], n // 3)
    rng = np.random.default_rng(4)
    idx = np.sort(rng.choice(n, 256, replace=False))
    D = eng.ml_descriptors(u, standardised=False)
    Do = np.array([LO.descriptor(u, L, i)[0] for i in idx])
    err = np.abs(D[idx] - Do) / (np.abs(Do) + np.abs(Do).mean(axis=0) + 1e-12)
    assert err.max() < 1e-4, err.max()
    E, F = eng.ml_labels(u)
    Eo, Fo = LO.labels_on(u, L, q, 0.650299, 0.3165492, nbg.workloads.K_EL, idx)
    assert S.rel_rmse(E[idx].astype(np.float64), Eo) < 5e-5
    assert S.rel_rmse(F[idx].astype(np.float64), Fo) < 5e-5
    th = [_random_params(21, D.astype(np.float64), E.astype(np.float64)),
          _random_params(22, D.astype(np.float64), E.astype(np.float64))]
    eng.ml_set_params(0, th[0])
    eng.ml_set_params(1, th[1])
    _, f_gpu = eng.ml_eval(u)
    sub = idx[::5][:48]
    f_o = LO.forces_on(u, L, [t.astype(np.float64) for t in th], sub)
    assert S.rel_rmse(f_gpu[sub], f_o) < 0.05, S.rel_rmse(f_gpu[sub], f_o)
    eng.close()
