"""Parity of the GPU rdf pair histogram (nbg_rdf_histogram) with the oracle's
restatement of the reference's loops (nbody_simulation_result.jl:664-709).
The counts are integers: every comparison is exact."""
import math

import numpy as np
import pytest

import systems as S

nbg = S.nbg
pytestmark = pytest.mark.gpu


def _hist(frames, idx, L, maxbin=1000):
    return nbg._abi.rdf_histogram(frames, idx, L, maxbin)


def _check(oracle, frames, idx, L, maxbin=1000):
    g = _hist(frames, idx, L, maxbin)
    o = oracle.rdf_histogram(frames, idx, L, maxbin)
    assert np.array_equal(g, o), f"{int(np.abs(g - o).sum())} counts differ in {int((g != o).sum())} bins"
    return g


def _lj_frames(n=1000, steps=200, every=10, seed=1):
    sim = S.lj_liquid(n, seed=seed)
    u0, v0 = S.state(sim)
    eng = sim.engine()
    _, _, tu, _, _ = eng.run(u0, v0, 0.005, steps, every)
    eng.close()
    return np.ascontiguousarray(np.stack(tu)), sim.boundary_conditions.L


@pytest.mark.parametrize("maxbin", [1000, 333])
def test_rdf_lj_trajectory(gpu, oracle, maxbin):
    frames, L = _lj_frames()
    g = _check(oracle, frames, np.arange(frames.shape[1]), L, maxbin)
    assert g.sum() > 0


def test_rdf_water_oxygens(gpu, oracle):
    sim = S.water_box(512, seed=4)
    u0, v0 = S.state(sim)
    eng = sim.engine()
    _, _, tu, _, _ = eng.run(u0, v0, 0.0005, 40, 10)
    eng.close()
    frames = np.ascontiguousarray(np.stack(tu))
    _check(oracle, frames, np.arange(0, frames.shape[1], 3), sim.boundary_conditions.L)


def test_rdf_bin_edges(gpu, oracle):
    """Distances at the bin edges k * dr and at L/2, where the FP32 screen
    hands the pairs to the reference's FP64 arithmetic; +-1 ulp dithers."""
    L, maxbin = 10.0, 1000
    dr = L / maxbin
    base = np.array([1.0, 2.0, 3.0])
    pts = [base]
    for k in range(1, 501):
        x = base[0] + k * dr
        pts += [np.array([x, base[1], base[2]]), np.array([np.nextafter(x, 0), base[1] + 0.0, base[2]]),
                np.array([np.nextafter(x, 20), base[1], base[2]])]
    for k in (1, 2, 57, 250, 353, 499, 500):  # diagonal edges
        c = k * dr / math.sqrt(3.0)
        pts.append(base + c)
    pts.append(base + np.array([0.5 * L, 0.0, 0.0]))  # exactly half the box
    pts.append(base - np.array([0.5 * L, 0.0, 0.0]))
    frame = np.array(pts)
    _check(oracle, frame[None], np.arange(len(frame)), L, maxbin)
    # the same distances shifted by whole boxes
    shifted = frame + L * np.random.default_rng(0).integers(-3, 4, size=frame.shape)
    _check(oracle, shifted[None], np.arange(len(frame)), L, maxbin)


def test_rdf_unwrapped_far(gpu, oracle):
    """Participants up to 200 boxes out: beyond 64 boxes their pairs all take
    the FP64 path, below it the FP32 screen."""
    frames, L = _lj_frames(n=500, steps=20, every=10, seed=2)
    rng = np.random.default_rng(5)
    shift = rng.integers(-200, 201, size=frames.shape) * (rng.random(frames.shape[:2])[..., None] < 0.3)
    _check(oracle, frames + L * shift, np.arange(frames.shape[1]), L)


@pytest.mark.parametrize("nidx", [0, 1, 2, 127, 128, 129, 300])
def test_rdf_ragged(gpu, oracle, nidx):
    rng = np.random.default_rng(nidx)
    L = 7.3
    frames = rng.uniform(-L, 2 * L, size=(3, max(nidx, 1) + 5, 3))
    idx = rng.permutation(frames.shape[1])[:nidx]
    g = _check(oracle, frames, idx, L)
    if nidx < 2:
        assert not g.any()


@pytest.mark.parametrize("maxbin", [1, 2, 16384])
def test_rdf_maxbin_limits(gpu, oracle, maxbin):
    rng = np.random.default_rng(maxbin)
    frames = rng.uniform(0, 3.0, size=(2, 400, 3))
    _check(oracle, frames, np.arange(400), 3.0, maxbin)


def test_rdf_no_frames(gpu):
    h = _hist(np.zeros((0, 10, 3)), np.arange(10), 2.0)
    assert h.shape == (1000,) and not h.any()


def test_rdf_errors(gpu):
    rng = np.random.default_rng(0)
    frames = rng.uniform(0, 2.0, size=(2, 50, 3))
    bad = frames.copy()
    bad[1, 7, 2] = np.nan
    with pytest.raises(nbg.EngineError) as e:
        _hist(bad, np.arange(50), 2.0)
    assert e.value.status == -4
    far = frames.copy()
    far[0, 3, 0] = 1e9
    with pytest.raises(nbg.EngineError) as e:
        _hist(far, np.arange(50), 2.0)
    assert e.value.status == -7
    for args in ((np.arange(50), 2.0, 0), (np.arange(50), 2.0, 16385), (np.array([0, 50]), 2.0, 10),
                 (np.arange(50), -1.0, 10)):
        with pytest.raises(nbg.EngineError) as e:
            _hist(frames, *args)
        assert e.value.status == -1
    # the histogram still works after the failed calls
    assert _hist(frames, np.arange(50), 2.0).sum() > 0


def test_rdf_device_buffers(gpu):
    torch = pytest.importorskip("torch")
    frames, L = _lj_frames(n=500, steps=20, every=10, seed=3)
    idx = np.arange(0, 500, 2)
    host = _hist(frames, idx, L)
    fd = torch.from_numpy(frames).cuda()
    out = torch.zeros(1000, dtype=torch.float64, device="cuda")
    nbg._abi.rdf_histogram(fd, idx, L, 1000, out=out)
    assert np.array_equal(out.cpu().numpy(), host)


def test_rdf_full_size_properties(gpu, oracle):
    """4096 oxygens of the 12,288-atom water box, 64 frames: additivity over
    frames, host (chunked upload) and device frames alike, invariance under a
    permutation of the participants, and two frames against the oracle."""
    pos, _, L = nbg.workloads.spcfw_water_box(4096, seed=7)
    rng = np.random.default_rng(9)
    frames = pos[None] + rng.normal(scale=0.02, size=(64,) + pos.shape)
    idx = np.arange(0, pos.shape[0], 3)
    full = _hist(frames, idx, L)  # host frames: uploaded in chunks, each chunk's kernels behind its copy
    halves = _hist(frames[:32], idx, L) + _hist(frames[32:], idx, L)
    assert np.array_equal(full, halves)
    torch = pytest.importorskip("torch")
    dev = nbg._abi.rdf_histogram(torch.from_numpy(frames).cuda(), idx, L, 1000)  # device frames: one launch
    assert np.array_equal(full, dev)
    assert np.array_equal(full, _hist(frames, rng.permutation(idx), L))
    assert full.sum() <= 64 * len(idx) * (len(idx) - 1)
    _check(oracle, frames[[0, 63]], idx, L)


def test_rdf_normalisation(gpu, oracle):
    """rdf(result): the GPU histogram with the reference's normalisation
    (nbody_simulation_result.jl:694-706)."""
    T, kb, sigma, m = 120.0, S.KB_KJ, 0.34, 39.95
    L = 5 * sigma
    bodies = nbg.generate_bodies_in_cell_nodes(125, m, math.sqrt(kb * T / m), L)
    system = nbg.PotentialNBodySystem(bodies, {"lennard_jones": nbg.LennardJonesParameters(T * kb, sigma, 0.5 * L)})
    sim = nbg.NBodySimulation(system, (0.0, 100 * 0.5e-3), nbg.CubicPeriodicBoundaryConditions(L), kb)
    res = nbg.run_simulation(sim, nbg.VelocityVerlet(), dt=0.5e-3, save_every=10)
    rs, gr = nbg.rdf(res)
    frames = np.stack(res.solution.u)
    hist = oracle.rdf_histogram(frames, np.arange(125), L, 1000)
    dr = L / 1000
    c = 4 / 3 * math.pi * 125 / L ** 3
    tlen = len(res.solution.t)
    for b in range(1000):
        rlower = b * dr
        nideal = c * ((rlower + dr) ** 3 - rlower ** 3)
        assert gr[b] == (hist[b] / (tlen * 125)) / nideal
        assert rs[b] == rlower + dr / 2
