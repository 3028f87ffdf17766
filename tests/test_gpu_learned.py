"""GPU tests of the learned short-range model and r-RESPA (through the C ABI):
descriptors, labels, BF16 forces and training gradients against the FP64
restatement in oracle/learned.py; GPU training; r-RESPA against velocity
Verlet, its fallback, and the ablation (trained network against none)."""
import math

import numpy as np
import pytest

import __graft_entry__ as g
import systems

pytestmark = pytest.mark.gpu

LO = g.load_learned_oracle()
N_MOL = 1000  # 3000 atoms, L = 3.10 nm: three list cells per side
K_EL = 138.935458
DT = 0.0005


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.sqrt(((a - b) ** 2).sum() / (b ** 2).sum()))


@pytest.fixture(scope="module")
def water(gpu):
    """An equilibrated box (2000 Berendsen steps at 300 K) and an engine with
    the learned model enabled."""
    sim, pos, vel, L = systems.spcfw_water_rf(N_MOL)
    eng = sim.engine()
    eng.set_state(pos, vel)
    eng.advance(DT, 2000)
    u, v = eng.get_state()
    eng.ml_enable()
    q = np.tile([-0.82, 0.41, 0.41], N_MOL)
    return dict(sim=sim, eng=eng, u=u, v=v, L=L, q=q)


@pytest.fixture(scope="module")
def trained(water):
    """The model trained on the GPU from 24 frames of the plain run (every 25
    steps), normalised on that set. Returns (theta_O, theta_H, losses, a held-out state)."""
    eng = water["eng"]
    eng.set_state(water["u"], water["v"])
    eng.ml_reserve(24)
    for _ in range(24):
        eng.advance(DT, 25)
        eng.ml_collect()
    eng.ml_normalize()
    eng.ml_init_params(seed=0, w1_scale=0.1)
    losses = [eng.ml_train(2500, batch=2048, lr=1e-3, seed=1), eng.ml_train(2500, batch=2048, lr=3e-4, seed=2)]
    eng.advance(DT, 200)
    held = eng.get_state()
    return eng.ml_get_params(0), eng.ml_get_params(1), losses, held


def _random_params(seed, D, E):
    rng = np.random.default_rng(seed)
    th = np.zeros(LO.n_params())
    th[:64 * 128] = 0.1 * rng.standard_normal(64 * 128) / 8
    o = 64 * 128 + 128
    th[o:o + 128 * 128] = rng.standard_normal(128 * 128) / math.sqrt(128)
    o2 = o + 128 * 128 + 128
    th[o2:o2 + 128] = rng.standard_normal(128) / math.sqrt(128)
    th[o2 + 128] = 0.3
    n = 24961
    th[n:n + 64] = D.mean(axis=0)
    th[n + 64:n + 128] = D.std(axis=0) + 1e-3
    th[n + 128], th[n + 129] = E.mean(), E.std()
    return th.astype(np.float32)


def test_descriptors_match_oracle(water):
    eng, u, L = water["eng"], water["u"], water["L"]
    D = eng.ml_descriptors(u, standardised=False)
    idx = list(range(0, len(u), 37))
    Do = np.array([LO.descriptor(u, L, i)[0] for i in idx])
    err = np.abs(D[idx] - Do) / (np.abs(Do) + np.abs(Do).mean(axis=0) + 1e-12)
    assert err.max() < 1e-4, err.max()


def test_labels_match_oracle(water):
    eng, u, L, q = water["eng"], water["u"], water["L"], water["q"]
    E, F = eng.ml_labels(u)
    Eo, Fo = LO.short_range_labels(u, L, q, 0.650299, 0.3165492, K_EL)
    assert rel(E, Eo) < 5e-5
    assert rel(F, Fo) < 5e-5


def test_training_gradient_matches_oracle(water):
    eng, u, L, q = water["eng"], water["u"], water["L"], water["q"]
    D = eng.ml_descriptors(u, standardised=False).astype(np.float64)
    E, _ = LO.short_range_labels(u, L, q, 0.650299, 0.3165492, K_EL)
    th = _random_params(11, D, E)
    eng.ml_set_params(0, th)
    rng = np.random.default_rng(5)
    X = rng.standard_normal((300, 64)).astype(np.float32)
    Y = rng.standard_normal(300).astype(np.float32)
    loss, grad = eng.ml_batch_gradient(0, X, Y)
    loss_o, grad_o = LO.train_gradients(th.astype(np.float64), X.astype(np.float64), Y.astype(np.float64))
    assert abs(loss - loss_o) < 1e-5 * abs(loss_o)
    assert rel(grad, grad_o) < 1e-5


def test_learned_forces_match_oracle_random_params(water):
    """BF16 tensor-core inference against the FP64 model with the same weights."""
    eng, u, L, q = water["eng"], water["u"], water["L"], water["q"]
    D = eng.ml_descriptors(u, standardised=False).astype(np.float64)
    E, _ = LO.short_range_labels(u, L, q, 0.650299, 0.3165492, K_EL)
    th = [_random_params(21, D, E), _random_params(22, D, E)]
    eng.ml_set_params(0, th[0])
    eng.ml_set_params(1, th[1])
    e_gpu, f_gpu = eng.ml_eval(u)
    e_o, f_o = LO.forces(u, L, [t.astype(np.float64) for t in th])
    assert rel(f_gpu, f_o) < 0.05
    assert abs(float(e_gpu.astype(np.float64).sum()) - e_o) < 0.01 * np.abs(E).sum()


def _mlp_energies(x, th):
    """Per-atom energies of the model on standardised descriptors, FP64."""
    th = th.astype(np.float64)
    w1 = th[:64 * 128].reshape(64, 128)
    o = 64 * 128
    b1 = th[o:o + 128]
    w2 = th[o + 128:o + 128 + 128 * 128].reshape(128, 128)
    o2 = o + 128 + 128 * 128
    b2, w3, b3 = th[o2:o2 + 128], th[o2 + 128:o2 + 256], th[o2 + 256]
    mu_e, sd_e = th[24961 + 128], th[24961 + 129]
    a2 = np.tanh(np.tanh(x @ w1 + b1) @ w2 + b2)
    return sd_e * (a2 @ w3 + b3) + mu_e


def test_mlp_tensor_memory_form_matches_warp_form(water, monkeypatch):
    """The MLP on tcgen05 with tensor-memory accumulators (NBG_MLP_TCGEN05)
    against the warp-level mma.sync form (the default) and the FP64 model on
    the same weights. Both forms round the products' inputs to BF16 and
    accumulate in FP32, so they agree to BF16 rounding; per-atom energies
    also match the FP64 network on the GPU's standardised descriptors."""
    eng, u, L, q = water["eng"], water["u"], water["L"], water["q"]
    D = eng.ml_descriptors(u, standardised=False).astype(np.float64)
    E, _ = LO.short_range_labels(u, L, q, 0.650299, 0.3165492, K_EL)
    th = [_random_params(31, D, E), _random_params(32, D, E)]
    eng.ml_set_params(0, th[0])
    eng.ml_set_params(1, th[1])
    e_ws, f_ws = eng.ml_eval(u)
    monkeypatch.setenv("NBG_MLP_TCGEN05", "1")
    e_tc, f_tc = eng.ml_eval(u)
    monkeypatch.delenv("NBG_MLP_TCGEN05")
    assert np.isfinite(e_tc).all() and np.isfinite(f_tc).all()
    assert rel(e_tc, e_ws) < 1e-2
    assert rel(f_tc, f_ws) < 1e-2
    x = eng.ml_descriptors(u, standardised=True).astype(np.float64)
    e_ref = np.where(np.arange(len(u)) % 3 == 0, _mlp_energies(x, th[0]), _mlp_energies(x, th[1]))
    assert rel(e_tc, e_ref) < 1e-2
    assert rel(e_ws, e_ref) < 1e-2
    e_o, f_o = LO.forces(u, L, [t.astype(np.float64) for t in th])
    assert rel(f_tc, f_o) < 0.05


def test_training_reaches_force_target(water, trained):
    thO, thH, losses, held = trained
    eng, L = water["eng"], water["L"]
    (lo0, lh0), (lo1, lh1) = losses
    assert lo1 < 1e-3 and lh1 < 1e-3, losses
    eng.ml_set_params(0, thO)
    eng.ml_set_params(1, thH)
    u = held[0]
    _, f_ml = eng.ml_eval(u)
    _, f_sr = eng.ml_labels(u)
    err = rel(f_ml, f_sr)
    assert err < 0.04, err
    # the GPU model is the FP64 model with these weights, to BF16 accuracy
    _, f_o = LO.forces(u, L, [thO.astype(np.float64), thH.astype(np.float64)])
    assert rel(f_ml, f_o) < 0.01


def test_respa_with_one_inner_step_is_velocity_verlet(water, trained):
    """Without a thermostat one inner step per outer step is velocity Verlet
    with the same total force, to rounding."""
    eng = _nve(water)
    eng.ml_set_params(0, trained[0])
    eng.ml_set_params(1, trained[1])
    u, v = trained[3]
    eng.set_state(u, v)
    eng.advance(DT, 20)
    ua, va = eng.get_state()
    eng.set_state(u, v)
    eng.respa_run(DT, 1, 20, threshold=0.0)
    ub, vb = eng.get_state()
    assert np.abs(ua - ub).max() < 1e-11
    assert np.abs(va - vb).max() < 1e-9


def _nve(water):
    sim, _, _, _ = systems.spcfw_water_rf(N_MOL, thermo=False)
    eng = sim.engine()
    eng.ml_enable()
    return eng


def _zero_output(theta):
    z = theta.copy()
    o = 64 * 128 + 128 + 128 * 128 + 128
    z[o:o + 129] = 0.0  # w3 and b3: E_i = mean_E, no learned force
    return z


def test_respa_ablation(water, trained):
    """Same start, NVE, 2 fs outer step (4 x 0.5 fs): the trained network
    keeps the energy close to velocity Verlet's; the split without it (fast
    force = bonded only) drifts far more. The r-RESPA error check measures
    the learned force against the exact short-range force every outer step."""
    thO, thH, _, held = trained
    eng = _nve(water)
    u, v = held
    e0 = eng.energy(u, v)["total"]
    n = len(u)

    def drift():
        uu, vv = eng.get_state()
        return abs(eng.energy(uu, vv)["total"] - e0) / n

    eng.set_state(u, v)
    eng.advance(DT, 800)
    d_vv = drift()
    eng.ml_set_params(0, thO)
    eng.ml_set_params(1, thH)
    eng.set_state(u, v)
    st = eng.respa_run(DT, 4, 200, threshold=0.0)
    d_ml = drift()
    assert st.outer_mts == 200 and st.outer_fallback == 0
    assert st.judge_mean < 0.04, st.judge_mean
    eng.set_state(u, v)
    eng.respa_run(DT, 4, 200, threshold=0.0, exact_split=True)
    d_exact = drift()
    eng.ml_set_params(0, _zero_output(thO))
    eng.ml_set_params(1, _zero_output(thH))
    eng.set_state(u, v)
    st0 = eng.respa_run(DT, 4, 200, threshold=0.0)
    d_zero = drift()
    assert st0.judge_mean > 0.99
    print(f"drift per atom over 400 fs: VV {d_vv:.3g}, exact split {d_exact:.3g}, learned {d_ml:.3g}, "
          f"no network {d_zero:.3g}")
    assert d_zero > 10 * d_ml, (d_zero, d_ml)
    assert d_ml < 2e-3, d_ml


def test_respa_judge_falls_back_to_velocity_verlet(water, trained):
    """With the untrained (zero-output) model every chunk fails the 2 % judge
    and is integrated again by velocity Verlet: the result is the plain run
    (up to the FP32 summation order of forces from lists rebuilt at other
    steps; an r-RESPA step with this model would differ by orders more)."""
    thO, thH, _, held = trained
    eng = _nve(water)
    u, v = held
    eng.ml_set_params(0, _zero_output(thO))
    eng.ml_set_params(1, _zero_output(thH))
    eng.set_state(u, v)
    st = eng.respa_run(DT, 4, 70, threshold=0.02)
    ub, vb = eng.get_state()
    assert st.outer_fallback == 70 and st.outer_mts == 0
    eng.set_state(u, v)
    eng.advance(DT, 64 * 4)
    eng.advance(DT, 6 * 4)
    ua, va = eng.get_state()
    assert np.abs(ua - ub).max() < 1e-6
    assert np.abs(va - vb).max() < 1e-4


def test_learned_api_errors(gpu):
    """The learned model refuses systems it does not model, and the r-RESPA
    entry point refuses bad arguments and unsupported thermostats."""
    import systems as S
    nbg = S.nbg
    # a Lennard-Jones liquid: not water
    sim = S.lj_liquid(1000, seed=2)
    eng = sim.engine()
    with pytest.raises(nbg.EngineError) as e:
        eng.ml_enable()
    assert e.value.status == -6  # NBG_ERR_UNSUPPORTED
    # calls before nbg_ml_enable
    sim, pos, vel, L = systems.spcfw_water_rf(1000)
    eng = sim.engine()
    with pytest.raises(nbg.EngineError):
        eng.ml_eval(pos)
    eng.ml_enable()
    with pytest.raises(nbg.EngineError):
        eng.ml_set_params(2, np.zeros(nbg._abi.NBG_ML_NPARAM, dtype=np.float32))
    with pytest.raises(nbg.EngineError):  # no resident state yet
        eng.respa_run(DT, 4, 1)
    eng.set_state(pos, vel)
    with pytest.raises(nbg.EngineError):
        eng.respa_run(-DT, 4, 1)
    with pytest.raises(nbg.EngineError):
        eng.respa_run(DT, 0, 1)
    with pytest.raises(nbg.EngineError):  # empty training set
        eng.ml_train(10)
    # Andersen is not supported by r-RESPA
    simA, pos, vel, L = systems.spcfw_water_rf(1000)
    simA.thermostat = nbg.AndersenThermostat(300.0, 10.0)
    engA = simA.engine()
    engA.ml_enable()
    engA.set_state(pos, vel)
    with pytest.raises(nbg.EngineError) as e:
        engA.respa_run(DT, 4, 1)
    assert e.value.status == -6


def test_thermostat_target_moves_temperature(water):
    """nbg_set_thermostat_target: a Berendsen run re-targeted to 320 K heats up."""
    sim, pos, vel, L = systems.spcfw_water_rf(1000)
    eng = sim.engine()
    eng.set_state(water["u"], water["v"])
    eng.set_thermostat_target(320.0)
    eng.advance(DT, 3000)
    u, v = eng.get_state()
    T = eng.energy(u, v)["temperature"]
    assert 305.0 < T < 335.0, T
