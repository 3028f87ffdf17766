#!/usr/bin/env python
"""Benchmark of the GB300 engine on the all-pairs gravity workload.

Workload (default): N = 65,536 equal-mass bodies (total mass 1, G = 1) from a
seeded Plummer sphere (scale radius 1), open boundaries, no softening,
velocity Verlet with dt = 1e-3. A step is one velocity-Verlet step of all
bodies (one all-pairs force evaluation). Metric: atom-steps/s.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference]
                  [--workload gravity|lj|water|ensemble|mts|rdf]

--workload mts (learned multiple-time-step water): 32,768 SPC/Fw molecules,
reaction field at 0.9 nm; the learned short-range model is trained on the GPU
from plain runs at 280, 300 and 320 K, then plain velocity Verlet (0.5 fs)
and r-RESPA (4 x 0.5 fs inner steps with the learned force, exact force every
2 fs) are timed side by side; metric ns/day.

value    : device-timed steps on the resident state (CUDA events on the
           engine's stream, L2 flushed between timed steps).
e2e      : the same steps through the reference-facing drop-in, nbg_accel
           on pinned host buffers (the SciML velocity-Verlet loop calling the
           GPU right-hand side, its update done in place on the host threads):
           every step uploads u (and v where the thermostat reads it) and
           reads back dv.
roofline : the dominant force kernel's algorithmic FLOP/s (20 flop per pair)
           or bytes against the measured peak. The LJ workload runs as
           persistent cluster launches of many steps: its line gives the step
           loop's time per step against the issue floor of the cluster's SMs
           (warp instructions per step from ncu), and the launch floor of the
           cluster shape. A batch that runs the persistent ensemble loop is
           reported the same way against all SMs; the ensemble tuner times
           the loop's forms and the per-step graphs after 100 untimed steps.
--workload rdf: the radial distribution function's pair histogram
(nbg_rdf_histogram, 1000 bins) over 512 frames of the 12,288-atom water box,
its 4096 oxygens (4.3e9 pair distances per step); metric pairs/s.

cpu_baseline : the FP64 oracle (a restatement of the reference's O(N^2)
           per-atom loops) on a bounded sample of the same step, host cores.
With --gpus N > 1 (torchrun) every rank runs its own replica: replicas only,
no collective on the data path.
"""
import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import __graft_entry__ as G  # noqa: E402

WORKLOADS = {
    "gravity": dict(name="gravity-plummer-65536", n=65536, dt=1e-3, steps=100),
    "lj": dict(name="lj-argon-1000", n=1000, dt=0.005, steps=1000),
    "water": dict(name="spcfw-water-12288", n=12288, dt=0.0005, steps=2000),
    "ensemble": dict(name="lj-langevin-ensemble-256", n=None, dt=0.005, steps=5000),
    "mts": dict(name="spcfw-water-98304-learned-respa", n=98304, dt=0.0005, steps=400),
    "rdf": dict(name="rdf-water-oxygens-4096x512", n=12288, dt=None, steps=20, frames=512, maxbin=1000),
}
RDF_FLOP_PER_PAIR = 40.0  # the FP32 screen of one pair (FMA = 2)
# SPC/Fw constants the water workloads run with, reported in their config
SPCFW_CONFIG = {"r0_nm": 0.1012, "theta0_deg": 113.24,
                "bond_k": "463700 kJ/mol/nm^2 (4637 read per square angstrom)", "angle_k": "383 kJ/mol/rad^2"}


class Workload:
    """Engine inputs of one benchmark workload: descriptors (one per replica),
    the initial state in the reference layout, and oracle descriptors."""

    def __init__(self, nbg, name, seed=0, n=None, rebuild_every=None, skin=None):
        self.name = name
        self.keep = []
        if name == "ensemble":
            reps = nbg.workloads.lj_ensemble(seed=seed)
            self.descs = []
            for r, rep in enumerate(reps):
                d, k = nbg.lennard_jones_descriptor(np.ones(rep["n"]), rep["L"],
                                                    thermostat=nbg.LangevinThermostat(rep["T"], 1.0),
                                                    seed=1000 + r, skin=ENS_SKIN if skin is None else skin,
                                                    rebuild_every=10 if rebuild_every is None else rebuild_every)
                # Euler-Maruyama (the reference's Langevin integrator) diverges
                # for an LJ liquid at dt = 0.005: BAOAB keeps velocity-Verlet stability
                d.flags |= nbg._abi.NBG_FLAG_LANGEVIN_BAOAB
                self.descs.append(d)
                self.keep.append(k)
            self.u0 = np.concatenate([rep["pos"] for rep in reps])
            self.v0 = np.concatenate([rep["vel"] for rep in reps])
            self.sizes = [rep["n"] for rep in reps]
        else:
            sim = make_sim(nbg, name, seed=seed, n=n, rebuild_every=rebuild_every, skin=skin)
            self.sim = sim
            d, k = nbg.system_descriptor(sim)
            self.descs = [d]
            self.keep.append(k)
            self.u0, self.v0, _ = nbg.gather_bodies_initial_coordinates(sim)
            self.sizes = [int(d.n)]
        self.n = int(sum(self.sizes))


def make_sim(nbg, workload, seed=0, n=None, rebuild_every=None, skin=None):
    if workload == "mts":
        return mts_sim(nbg, (n or WORKLOADS["mts"]["n"]) // 3, seed=seed)[0]
    if workload == "gravity":
        pos, vel, m = nbg.workloads.plummer_sphere(n or 65536, seed=seed)
        bodies = [nbg.MassBody(pos[i], vel[i], m[i]) for i in range(len(m))]
        return nbg.NBodySimulation(nbg.GravitationalSystem(bodies, 1.0), (0.0, 0.1))
    if workload == "lj":
        pos, vel, L = nbg.workloads.lj_argon_lattice(1000, rho=0.8, T=1.0, seed=seed)
        bodies = [nbg.MassBody(pos[i], vel[i], 1.0) for i in range(len(pos))]
        sysm = nbg.PotentialNBodySystem(bodies, {"lennard_jones": nbg.LennardJonesParameters(1.0, 1.0, 2.5)})
        return nbg.NBodySimulation(sysm, (0.0, 5.0), nbg.CubicPeriodicBoundaryConditions(L), kb=1.0, skin=0.3,
                                   rebuild_every=10 if rebuild_every is None else rebuild_every)
    if workload == "water":
        pos, vel, L = nbg.workloads.spcfw_water_box(4096, seed=seed, T=300.0)
        bodies = nbg.workloads.water_molecules(pos, vel)
        lj = nbg.LennardJonesParameters(0.650299, 0.3165492, 0.9)
        el = nbg.ElectrostaticParameters(nbg.workloads.K_EL, 0.9)
        spc = nbg.SPCFwParameters(0.1012, 113.24 * math.pi / 180, nbg.workloads.SPCFW_KB, nbg.workloads.SPCFW_KA)
        water = nbg.WaterSPCFw(bodies, nbg.workloads.M_H, nbg.workloads.M_O, 0.41, -0.82, lj, el, spc)
        return nbg.NBodySimulation(water, (0.0, 1.0), nbg.CubicPeriodicBoundaryConditions(L),
                                   nbg.BerendsenThermostat(300.0, 0.1), kb=nbg.workloads.KB_KJ,
                                   skin=0.1 if skin is None else skin,
                                   rebuild_every=WATER_REBUILD if rebuild_every is None else rebuild_every)
    raise ValueError(workload)


# The replica batch's list skin (its configuration leaves the list to the
# engine): with the 10-step rebuild period, 0.5 sigma makes the displacement
# trigger rare between the periodic rebuilds of all replicas at once, at 23 %
# more list entries than 0.3 (0.697 -> 0.621 ms per step over 2000 steps;
# 0.6: 0.651, 0.5 with periods of 15 or 20 or on displacement only: 0.72-0.79).
ENS_SKIN = 0.5

# The water workloads rebuild their Verlet lists only when an atom moved
# more than skin/2 (the lists stay supersets of the exact pair set either
# way): with 0.1 nm of skin at 300 K the fixed 10-step period rebuilt them
# several times more often than needed (12k water 70.7 -> 64.5 us per step,
# 98k water 172 -> 186 ns/day). The LJ workloads keep the 10-step period:
# LJ-1000's configuration states it, and for the replica batch it is the
# faster schedule (0.697 against 0.718 ms per step).
WATER_REBUILD = 0

# the ensemble tuner's window: ENS_TUNE_STEPS steps per form, from the state
# after ENS_TUNE_AFTER untimed steps
ENS_TUNE_AFTER = 100
ENS_TUNE_STEPS = 20


def algorithmic_work(workload, n, eng):
    """(amount per force-kernel launch, unit, bound) from the per-unit figures:
    gravity 20 flop per ordered pair; list kernels the bytes a launch must move."""
    if workload == "gravity":
        return 20.0 * n * (n - 1), "TFLOP/s", "fp32"
    # the fixed-point list kernel: per atom its 16 B position record (each
    # neighbour's gather counted once per atom in HBM terms) + 24 B acceleration
    # write + 4 B per list entry
    nbr = 419.0 if workload == "water" else 73.6  # water: 1.0 nm list; LJ liquids (single and ensemble): 2.8 sigma
    return n * (16 + 24 + 4 * nbr), "GB/s", "hbm"


class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.proc = None
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            p = [x.strip() for x in line.split(",")]
            if len(p) < 8:
                continue
            try:
                sm.append(float(p[0]))
                smax.append(float(p[1]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if p[4 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except OSError:
        return {}


def profile_value(kernel, table="traffic.json"):
    """A per-launch figure of `kernel` from a committed ncu summary table, if
    any: traffic.json holds DRAM bytes, issue.json warp instructions."""
    path = os.path.join(ROOT, "profiles", table)
    try:
        with open(path) as f:
            return json.load(f).get(kernel)
    except (OSError, ValueError):
        return None


def profile_traffic(kernel):
    return profile_value(kernel)


def cpu_baseline(oracle, wl, target_s=8.0):
    """The oracle on a bounded sample of one step, on every host core:
    accelerations of a subset of atoms over all their partners (the
    reference's per-atom loops), atom-steps/s = atoms / time. For the ensemble,
    a stratified sample of replicas, timed whole, fitted to c N^2 and summed
    over all replicas (the reference's cost is all-pairs per replica)."""
    cores = os.cpu_count() or 1
    oracle.set_threads(cores)
    if wl.name == "ensemble":
        order = np.argsort(wl.sizes)
        pick = order[np.linspace(0, len(order) - 1, 6).astype(int)]
        offs = np.concatenate([[0], np.cumsum(wl.sizes)])
        cs, done, el = [], 0, 0.0
        for r in pick:
            u = wl.u0[offs[r]:offs[r + 1]]
            t0 = time.perf_counter()
            oracle.partial_accel(wl.descs[r], u, 0, wl.sizes[r])
            dt = time.perf_counter() - t0
            cs.append(dt / wl.sizes[r] ** 2)
            done += wl.sizes[r]
            el += dt
        c = float(np.mean(cs))
        step_s = c * float(np.sum(np.asarray(wl.sizes, dtype=np.float64) ** 2))
        return {"value": wl.n / step_s, "unit": "atom-steps/s", "cores": cores, "kind": "port",
                "sample": f"{len(pick)} replicas (sizes {sorted(int(wl.sizes[r]) for r in pick)}) timed whole, "
                          f"{el:.1f} s; step time = c * sum N_r^2 over all {len(wl.sizes)} replicas"}
    desc, u, n = wl.descs[0], wl.u0, wl.n
    i1 = min(n, 64)
    t0 = time.perf_counter()
    oracle.partial_accel(desc, u, 0, i1)
    per_atom = (time.perf_counter() - t0) / i1
    k = int(max(i1, min(n, target_s / max(per_atom, 1e-9))))
    reps = min(20, max(1, int(target_s / max(per_atom * k, 1e-9))))
    t0 = time.perf_counter()
    done = 0
    for r in range(reps):
        s0 = (r * k) % n
        s1 = min(n, s0 + k)
        oracle.partial_accel(desc, u, s0, s1)
        done += s1 - s0
    el = time.perf_counter() - t0
    all_cores = done / el
    oracle.set_threads(1)
    m = max(8, min(n, int(2.0 / max(per_atom * cores, 1e-9))))
    t0 = time.perf_counter()
    oracle.partial_accel(desc, u, 0, m)
    one = m / (time.perf_counter() - t0)
    return {"value": all_cores, "unit": "atom-steps/s", "cores": cores, "kind": "port",
            "sample": f"{done} atom force evaluations (all {n} partners each) in {reps} slices, "
                      f"{el:.1f} s wall; one step = {n} atoms",
            "value_1thread": one, "sample_1thread": f"{m} atoms on 1 thread"}


def rdf_frames(nbg, n_atoms, nframes, seed=0, step_nm=0.01):
    """A trajectory of the SPC/Fw water box (n_atoms / 3 molecules at
    0.997 g/cm^3): frame 0 is the seeded lattice, later frames add a Gaussian
    random walk of step_nm per coordinate and frame (unwrapped positions).
    Returns (frames (nframes, n_atoms, 3), oxygen columns, L)."""
    pos, _, L = nbg.workloads.spcfw_water_box(n_atoms // 3, seed=seed)
    rng = np.random.default_rng(seed + 1)
    frames = np.empty((nframes,) + pos.shape)
    frames[0] = pos
    for f in range(1, nframes):
        frames[f] = frames[f - 1] + rng.normal(scale=step_nm, size=pos.shape)
    return frames, np.arange(0, pos.shape[0], 3, dtype=np.int32), L


def rdf_cpu_rate(oracle, frames, idx, L, maxbin, target_s):
    """The oracle's histogram on whole frames until target_s has passed:
    (pairs/s, frames done, seconds)."""
    npairs = len(idx) * (len(idx) - 1) // 2
    done, t0 = 0, time.perf_counter()
    while True:
        oracle.rdf_histogram(frames[done % len(frames)][None], idx, L, maxbin)
        done += 1
        el = time.perf_counter() - t0
        if el >= target_s:
            return done * npairs / el, done, el


def run_reference(args, rank):
    """--impl reference: the oracle's restatement of the reference's O(N^2)
    per-atom loops on the host cores, each step a bounded sample of the
    workload's force evaluation (atoms over all partners)."""
    if rank != 0:
        return
    nbg = G.load_package()
    oracle = G.load_oracle()
    w = WORKLOADS[args.workload]
    if args.workload == "rdf":
        # each step: the reference rdf's pair loops over `ref_frames` whole frames
        frames, idx, L = rdf_frames(nbg, w["n"], w["frames"])
        cores = os.cpu_count() or 1
        oracle.set_threads(cores)
        npairs = len(idx) * (len(idx) - 1) // 2
        k = args.ref_frames
        for s in range(args.warmup):
            oracle.rdf_histogram(frames[s % len(frames)][None], idx, L, w["maxbin"])
        t0 = time.perf_counter()
        for s in range(args.steps):
            f0 = (s * k) % len(frames)
            oracle.rdf_histogram(frames[f0:f0 + k], idx, L, w["maxbin"])
        el = time.perf_counter() - t0
        val = args.steps * k * npairs / el
        sample = (f"{k} whole frame(s) per step ({len(idx)} oxygens, {npairs} pairs each) of the "
                  f"{w['frames']}-frame trajectory: the FP64 restatement of the reference rdf's loops")
        line = {"metric": "rdf pairs/s", "value": val, "unit": "pairs/s", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded lattice + random walk)", "impl": "reference",
                "config": {"workload": w["name"], "atoms": w["n"], "participants": len(idx),
                           "frames": w["frames"], "maxbin": w["maxbin"], "sample_frames_per_step": k},
                "cpu_baseline": {"value": val, "unit": "pairs/s", "cores": cores, "kind": "port", "sample": sample},
                "e2e": {"value": val, "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    wl = Workload(nbg, args.workload, n=args.n, rebuild_every=args.rebuild_every)
    cores = os.cpu_count() or 1
    oracle.set_threads(cores)
    offs = np.concatenate([[0], np.cumsum(wl.sizes)])

    def sample_step(s):
        """one bounded sample: `ref_sample` atoms of one system / replica"""
        r = s % len(wl.sizes)
        n_r = wl.sizes[r]
        a = (s * args.ref_sample) % n_r
        b = min(n_r, a + args.ref_sample)
        oracle.partial_accel(wl.descs[r], wl.u0[offs[r]:offs[r + 1]], a, b)
        return b - a

    for s in range(args.warmup):
        sample_step(s)
    t0 = time.perf_counter()
    done = 0
    for s in range(args.steps):
        done += sample_step(s)
    el = time.perf_counter() - t0
    val = done / el
    if wl.name == "ensemble":
        # all-pairs cost grows with N_r: rescale the sampled rate to the ensemble's mix
        sz = np.asarray(wl.sizes, dtype=np.float64)
        sampled = np.asarray([wl.sizes[s % len(sz)] for s in range(args.steps)], dtype=np.float64)
        val = val * sampled.mean() / (np.sum(sz ** 2) / np.sum(sz))
    line = {"metric": "atom-steps/s", "value": val, "unit": "atom-steps/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * wl.n / val,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded)", "impl": "reference",
            "config": {"workload": w["name"], "N": wl.n, "dt": w["dt"], "sample_atoms_per_step": args.ref_sample},
            "cpu_baseline": {"value": val, "unit": "atom-steps/s", "cores": cores, "kind": "port",
                             "sample": f"{args.ref_sample} atoms' forces per step over all partners "
                                       "(the FP64 restatement of the reference's per-atom loops)"},
            "e2e": {"value": val, "unit": "atom-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def max_over_ranks(value, dist, device):
    """The largest of every rank's `value` (the job's time is its slowest
    rank's); `value` itself without a process group."""
    if dist is None:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def mts_sim(nbg, n_mol, thermo=True, T=300.0, seed=0, rebuild_every=None):
    """SPC/Fw water (benchmark parameters), reaction field (eps_rf 78.5) at 0.9 nm."""
    pos, vel, L = nbg.workloads.spcfw_water_box(n_mol, seed=seed, T=T)
    bodies = nbg.workloads.water_molecules(pos, vel)
    lj = nbg.LennardJonesParameters(0.650299, 0.3165492, 0.9)
    el = nbg.ElectrostaticParameters(nbg.workloads.K_EL, 0.9, 78.5)
    spc = nbg.SPCFwParameters(0.1012, 113.24 * math.pi / 180, nbg.workloads.SPCFW_KB, nbg.workloads.SPCFW_KA)
    water = nbg.WaterSPCFw(bodies, nbg.workloads.M_H, nbg.workloads.M_O, 0.41, -0.82, lj, el, spc)
    th = nbg.BerendsenThermostat(T, 0.1) if thermo else nbg.NullThermostat()
    sim = nbg.NBodySimulation(water, (0.0, 1.0), nbg.CubicPeriodicBoundaryConditions(L), th,
                              kb=nbg.workloads.KB_KJ, skin=0.1,
                              rebuild_every=WATER_REBUILD if rebuild_every is None else rebuild_every)
    return sim, pos, vel


def run_mts(args, rank, world):
    """Learned multiple-time-step water: train, then time plain velocity
    Verlet against learned and exact-split r-RESPA on one equilibrated state."""
    import torch
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    device = torch.cuda.current_device()
    nbg = G.load_package()
    nbg.load_library()
    w = WORKLOADS["mts"]
    n_mol = (args.n or w["n"]) // 3
    dt, inner = w["dt"], 4
    outer = max(1, args.steps // inner)
    K = outer * inner
    sim, pos, vel = mts_sim(nbg, n_mol, seed=rank, rebuild_every=args.rebuild_every)
    n = 3 * n_mol
    eng = sim.engine()
    # a stream of torch's, current for the flush and the events, on which
    # the library launches (its handle is not the legacy default stream's 0,
    # which nbg_set_stream would read as "the context's own stream")
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    eng.set_stream(stream.cuda_stream)
    eng.set_state(pos, vel)
    t_setup = time.perf_counter()
    eng.advance(dt, 4000)  # equilibration from the contact-free lattice start (2 ps)
    # training data: plain runs at 280, 300 and 320 K, 8 frames each (every 100 steps after 1000)
    eng.ml_enable()
    frames_per_T, temps = 8, (280.0, 300.0, 320.0)
    eng.ml_reserve(frames_per_T * len(temps))
    for T in temps:
        eng.set_thermostat_target(T)
        eng.advance(dt, 1000)
        for _ in range(frames_per_T):
            eng.advance(dt, 100)
            rows = eng.ml_collect()
    eng.set_thermostat_target(300.0)
    eng.ml_normalize()
    eng.ml_init_params(seed=0, w1_scale=0.1)
    torch.cuda.synchronize()
    t_train = time.perf_counter()
    loss1 = eng.ml_train(args.train_steps, batch=2048, lr=1e-3, seed=1)
    loss2 = eng.ml_train(args.train_steps, batch=2048, lr=3e-4, seed=2)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t_train
    eng.advance(dt, 1000)  # back at 300 K; a state none of the frames saw
    u0, v0 = eng.get_state()
    tuned = eng.autotune(5)  # lanes per atom of the exact non-bonded force
    _, f_ml = eng.ml_eval(u0)
    _, f_sr = eng.ml_labels(u0)
    f_sr = f_sr.astype(np.float64)
    force_rmse = float(np.linalg.norm(f_ml - f_sr) / np.linalg.norm(f_sr))
    ml_ms = eng.ml_kernel_times(10)
    t_setup = time.perf_counter() - t_setup

    def timed(fn):
        eng.set_state(u0, v0)
        fn(args.warmup)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        l0 = eng.kernel_launches
        torch.cuda.nvtx.range_push("timed")
        e0.record(stream)
        res = fn(None)
        e1.record(stream)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        return e0.elapsed_time(e1), eng.kernel_launches - l0, res

    sampler = ClockSampler(device)
    ms_plain, l_plain, _ = timed(lambda warm: eng.advance(dt, K if warm is None else warm))
    ms_ml, l_ml, st_ml = timed(lambda warm: eng.respa_run(dt, inner, outer if warm is None else warm, 0.02))
    ms_ex, l_ex, _ = timed(lambda warm: eng.respa_run(dt, inner, outer if warm is None else warm, 0.0,
                                                        exact_split=True))
    # the scheme's own cost: the same outer steps with no fast non-bonded
    # force at all (bonded terms only), the ceiling of any fast model here
    ms_sk, l_sk, _ = timed(lambda warm: eng.respa_run(dt, inner, outer if warm is None else warm, 0.0,
                                                        no_fast_force=True))
    clocks = sampler.stop()
    fs_per_day = lambda ms, fs: fs / (ms / 1e3) * 86400 / 1e6  # ns/day
    ns_plain = fs_per_day(ms_plain, K * dt * 1e3)
    ns_ml = fs_per_day(ms_ml, K * dt * 1e3)
    ns_ex = fs_per_day(ms_ex, K * dt * 1e3)
    ns_sk = fs_per_day(ms_sk, K * dt * 1e3)

    # end to end through the public call: host state in, r-RESPA, host state out
    uh = torch.from_numpy(u0).pin_memory().numpy()
    vh = torch.from_numpy(v0).pin_memory().numpy()
    t0 = time.perf_counter()
    eng.set_state(uh, vh)
    eng.respa_run(dt, inner, outer, 0.02)
    ue, ve = eng.get_state()
    e2e_s = time.perf_counter() - t0

    # energy drift, NVE, 1 ps from the same state: velocity Verlet against learned r-RESPA
    simN, _, _ = mts_sim(nbg, n_mol, thermo=False, seed=rank, rebuild_every=args.rebuild_every)
    en = simN.engine()
    en.ml_enable()
    en.ml_set_params(0, eng.ml_get_params(0))
    en.ml_set_params(1, eng.ml_get_params(1))
    e_0 = en.energy(u0, v0)["total"]
    drift = {}
    for name, fn in (("plain", lambda: en.advance(dt, 2000)), ("learned_respa", lambda: en.respa_run(dt, inner, 500, 0.0)),
                     ("exact_split_respa", lambda: en.respa_run(dt, inner, 500, 0.0, exact_split=True))):
        en.set_state(u0, v0)
        fn()
        uu, vv = en.get_state()
        drift[name] = (en.energy(uu, vv)["total"] - e_0) / n / 1e-3  # kJ/mol per atom per ns
    peaks = measured_peaks()
    flop_atom = 2 * (64 * 128 + 128 * 128 + 128) + 2 * (128 * 128 + 64 * 128)  # forward + backward to the inputs
    achieved = flop_atom * n / (ml_ms[2] / 1e3) / 1e12
    peak = peaks.get("bf16_tflops")
    line = {"metric": "ns/day (learned r-RESPA)", "value": ns_ml, "unit": "ns/day", "n_gpus": world,
            "steps": K, "warmup": args.warmup, "ms_per_step": ms_ml / K, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "bf16 MLP (fp32 accumulate), f32 pair forces, f64 state",
            "data": "synthetic (seeded generator, no dataset); training frames from this run's plain MD",
            "config": {"workload": w["name"], "N": n, "dt_inner_fs": dt * 1e3, "inner_steps": inner,
                       "dt_outer_fs": dt * inner * 1e3, "electrostatics": "reaction field eps_rf 78.5, 0.9 nm",
                       "spcfw": SPCFW_CONFIG,
                       "thermostat": "Berendsen 300 K tau 0.1 ps", "l2": "no flush (state L2-resident across steps)",
                       "lanes_per_atom": tuned[0], "autotune_force_ms": tuned[1],
                       "training": {"frames": frames_per_T * len(temps), "temperatures_K": list(temps),
                                    "atom_environments": list(rows), "adam_steps_per_species": 2 * args.train_steps, "batch": 2048,
                                    "final_loss_std_units": list(loss2), "train_s": t_train}},
            "plain_ns_per_day": ns_plain, "exact_split_ns_per_day": ns_ex,
            "speedup_vs_plain": ns_ml / ns_plain, "exact_split_speedup_vs_plain": ns_ex / ns_plain,
            "no_fast_force_ns_per_day": ns_sk, "no_fast_force_speedup_vs_plain": ns_sk / ns_plain,
            "ms_per_outer_step": {"plain_4_steps": 4 * ms_plain / K, "learned": inner * ms_ml / K,
                                  "exact_split": inner * ms_ex / K, "no_fast_force": inner * ms_sk / K},
            "atom_steps_per_s": {"plain": n * K / (ms_plain / 1e3), "learned_respa": n * K / (ms_ml / 1e3),
                                 "exact_split_respa": n * K / (ms_ex / 1e3)},
            "learned_force_rel_rmse": force_rmse,
            "judge": {"mean": st_ml.judge_mean, "max": st_ml.judge_max, "outer_mts": st_ml.outer_mts,
                      "outer_fallback": st_ml.outer_fallback, "threshold": 0.02},
            "energy_drift_kj_mol_atom_ns": drift,
            "ml_kernel_ms": {"short_list": ml_ms[0], "descriptors": ml_ms[1], "mlp_bf16": ml_ms[2],
                             "force_scatter": ml_ms[3]},
            "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak if peak else None,
                         "traffic": profile_traffic(f"k_mlp_bf16:{w['name']}"), "kernel": "k_mlp_bf16",
                         "kernel_ms": ml_ms[2], "peak_source": "measured" if peak else None},
            "e2e": {"value": n * K / e2e_s, "unit": "atom-steps/s", "h2d_bytes_per_step": 2 * uh.nbytes / K,
                    "d2h_bytes_per_step": 2 * uh.nbytes / K,
                    "path": "nbg_set_state + nbg_respa_run + nbg_get_state from pinned host buffers"},
            "gpu_launches": l_ml, "clocks": clocks, "setup_s": t_setup}
    if rank == 0 and world == 1 and not args.no_cpu:
        oracle = G.load_oracle()

        class _W:
            pass
        wl = _W()
        d, k = nbg.system_descriptor(sim)
        wl.name, wl.descs, wl.u0, wl.n, wl.keep = "mts", [d], u0, n, k
        line["cpu_baseline"] = cpu_baseline(oracle, wl)
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_rdf(args, rank, world):
    """The radial distribution function's pair histogram over a trajectory:
    one step = nbg_rdf_histogram over all frames (every replica its own)."""
    import torch
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    device = local
    nbg = G.load_package()
    lib = nbg.load_library()
    w = WORKLOADS["rdf"]
    maxbin = w["maxbin"]
    frames, idx, L = rdf_frames(nbg, w["n"], w["frames"], seed=rank)
    npairs = w["frames"] * (len(idx) * (len(idx) - 1) // 2)
    hist = lambda fr, out: nbg._abi.rdf_histogram(fr, idx, L, maxbin, device, out=out)
    fd = torch.from_numpy(frames).to(f"cuda:{device}")
    out = torch.zeros(maxbin, dtype=torch.float64, device=f"cuda:{device}")
    pk = ctypes.c_double()
    peak = pk.value if lib.nbg_probe_fp32_peak(device, ctypes.byref(pk)) == 0 else None
    for _ in range(args.warmup):
        hist(fd, out)
    ref_hist = out.cpu().numpy().copy()
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{device}")
    stream = torch.cuda.current_stream()  # the legacy default stream, where the library launches
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(device)
    step_ms, pair_ms, pack_ms = [], [], []
    torch.cuda.nvtx.range_push("timed")
    for s in range(args.steps):
        flush.fill_(float(s))
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        hist(fd, out)
        e1.record(stream)
        torch.cuda.synchronize()
        step_ms.append(e0.elapsed_time(e1))
        km = nbg._abi.rdf_kernel_times()
        pack_ms.append(km[0])
        pair_ms.append(km[1])
    torch.cuda.nvtx.range_pop()
    clocks = sampler.stop()
    total_ms = max_over_ranks(float(sum(step_ms)), dist, f"cuda:{device}")
    value = npairs * args.steps * world / (total_ms / 1e3)
    deterministic = bool(np.array_equal(out.cpu().numpy(), ref_hist))

    e2e = None
    if not args.no_e2e:
        # the public call on host buffers: frames uploaded, histogram read back, every step
        fh = torch.from_numpy(frames).pin_memory()
        hh = torch.zeros(maxbin, dtype=torch.float64).pin_memory()
        fhn, hhn = fh.numpy(), hh.numpy()
        hist(fhn, hhn)
        e2e_steps = max(3, min(args.steps, 20))
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            hist(fhn, hhn)
        e2e_s = time.perf_counter() - t0
        deterministic = deterministic and bool(np.array_equal(hhn, ref_hist))
        e2e = {"value": npairs * e2e_steps * world / e2e_s, "unit": "pairs/s", "h2d_bytes_per_step": fhn.nbytes,
               "d2h_bytes_per_step": hhn.nbytes + 8,
               "path": "nbg_rdf_histogram on pinned host frames (all columns uploaded, histogram and status read back)",
               "steps": e2e_steps}

    pairs_kernel_ms = statistics.mean(pair_ms)
    achieved = npairs * RDF_FLOP_PER_PAIR / (pairs_kernel_ms / 1e3) / 1e12
    line = {"metric": "rdf pairs/s", "value": value, "unit": "pairs/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 screen, f64 (the reference's arithmetic) for pairs near a bin edge; integer counts",
            "data": "synthetic (seeded water lattice + Gaussian random walk, unwrapped)",
            "config": {"workload": w["name"], "atoms": w["n"], "participants": len(idx), "frames": w["frames"],
                       "maxbin": maxbin, "L_nm": L, "l2": "512 MB buffer written between timed steps (L2 flushed)",
                       "parallelism": "replicas only" if world > 1 else "single GPU"},
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak if peak else None,
                         "traffic": profile_traffic(f"k_rdf_pairs:{w['name']}"), "kernel": "k_rdf_pairs",
                         "kernel_ms": pairs_kernel_ms, "kernel_launches": args.steps,
                         "flop_per_pair": RDF_FLOP_PER_PAIR,
                         "peak_source": "FP32 FMA probe measured in this run (nbg_probe_fp32_peak)"},
            "split_kernel_ms": statistics.mean(pack_ms), "e2e": e2e, "gpu_launches": 3 * args.steps,
            "clocks": clocks, "histogram_repeatable": deterministic}
    if rank == 0 and world == 1 and not args.no_cpu:
        oracle = G.load_oracle()
        cores = os.cpu_count() or 1
        oracle.set_threads(cores)
        # parity on two frames, then the oracle's rate on whole frames
        pick = [0, w["frames"] - 1]
        gsub = nbg._abi.rdf_histogram(frames[pick], idx, L, maxbin, device)
        line["parity_two_frames_exact"] = bool(np.array_equal(gsub, oracle.rdf_histogram(frames[pick], idx, L,
                                                                                          maxbin)))
        rate, done, el = rdf_cpu_rate(oracle, frames, idx, L, maxbin, 10.0)
        oracle.set_threads(1)
        rate1, done1, el1 = rdf_cpu_rate(oracle, frames, idx, L, maxbin, 3.0)
        oracle.set_threads(cores)
        line["cpu_baseline"] = {"value": rate, "unit": "pairs/s", "cores": cores, "kind": "port",
                                "sample": f"{done} whole frames ({len(idx)} oxygens each) in {el:.1f} s: the FP64 "
                                          "restatement of the reference rdf's loops",
                                "value_1thread": rate1, "sample_1thread": f"{done1} whole frames on 1 thread"}
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--workload", default="gravity", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--no-flush", action="store_true", help="time all steps back to back (no L2 flush)")
    ap.add_argument("--skin", type=float, default=None,
                    help="Verlet-list skin of the replica batch or the 12k water box (defaults 0.5 sigma, 0.1 nm)")
    ap.add_argument("--rebuild-every", type=int, default=None,
                    help="Verlet-list rebuild period of the list workloads (0: only when an atom moved more than "
                         "skin/2; default: the workload's own)")
    ap.add_argument("--ref-sample", type=int, default=2048)
    ap.add_argument("--ref-frames", type=int, default=16, help="rdf: whole frames per reference step")
    ap.add_argument("--save-every", type=int, default=0,
                    help="also time nbg_run with trajectory frames every N steps (single systems)")
    ap.add_argument("--n", type=int, default=None, help="gravity body count (smaller profiling captures)")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg")
    ap.add_argument("--grav-plain", action="store_true", help="gravity with plain FP32 positions")
    ap.add_argument("--train-steps", type=int, default=4000,
                    help="mts: Adam steps per species in each of the two training phases")
    args = ap.parse_args()
    w = WORKLOADS[args.workload]
    if args.steps is None:
        args.steps = w["steps"]
    if args.warmup < 3:
        args.warmup = 3

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist_mod
        dist = dist_mod
    if args.impl == "reference":
        run_reference(args, rank)
        return

    import torch
    if dist is not None:
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    if args.workload in ("mts", "rdf"):
        (run_mts if args.workload == "mts" else run_rdf)(args, rank, world)
        if dist is not None:
            dist.destroy_process_group()
        return
    torch.cuda.set_device(local)
    device = local
    nbg = G.load_package()
    nbg.load_library()
    wl = Workload(nbg, args.workload, seed=rank, n=args.n, rebuild_every=args.rebuild_every, skin=args.skin)
    if args.grav_plain:
        wl.descs[0].flags |= nbg._abi.NBG_FLAG_GRAV_PLAIN
    u0, v0, n = wl.u0, wl.v0, wl.n
    dt = w["dt"]
    eng = nbg.Engine(wl.descs, device)
    # a stream of torch's, current for the flush and the events, on which
    # the library launches (nbg_advance returns without waiting, so the
    # events must be on the library's stream; the legacy default stream's
    # handle 0 would select the context's own stream)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    eng.set_stream(stream.cuda_stream)
    batch = len(wl.descs) > 1
    # the ensemble's working set (~0.5 GB) exceeds L2 by itself
    flush_steps = not args.no_flush and not batch

    peak_fp32 = None
    if args.workload == "gravity":
        pk = ctypes.c_double()
        if eng.lib.nbg_probe_fp32_peak(device, ctypes.byref(pk)) == 0:
            peak_fp32 = pk.value

    eng.set_state(u0, v0)
    e_start = None if batch else eng.energy(u0, v0)
    tuned = None
    ens_tuned = None
    if args.workload in ("lj", "water", "ensemble"):
        # the list force kernel's lanes per atom, timed on this state (untimed here)
        tuned = eng.autotune(5)
    if batch and eng.ensemble_form() is not None:
        # the persistent ensemble loop's form (lanes, threads per replica,
        # cell width) or the per-step graphs, timed (untimed here) once the
        # lattice has melted: in its first steps the replicas rarely rebuild
        # their lists, which favours the loop over what follows
        eng.advance(dt, ENS_TUNE_AFTER)
        ens_tuned = eng.ensemble_tune(ENS_TUNE_STEPS)
    eng.advance(dt, args.warmup)
    torch.cuda.synchronize()
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{device}")

    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(device)
    launches0 = eng.kernel_launches
    step_ms = []
    torch.cuda.nvtx.range_push("timed")  # ncu --nvtx --nvtx-include timed/ captures this region
    if not flush_steps:
        # all K steps back to back (the step loop replays captured CUDA graphs)
        flush.fill_(0.0)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        eng.advance(dt, args.steps)
        e1.record(stream)
        torch.cuda.synchronize()
        step_ms = [e0.elapsed_time(e1) / args.steps] * args.steps
    else:
        for s in range(args.steps):
            flush.fill_(float(s))
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            eng.advance(dt, 1)
            e1.record(stream)
            torch.cuda.synchronize()
            step_ms.append(e0.elapsed_time(e1))
    torch.cuda.nvtx.range_pop()
    launches = eng.kernel_launches - launches0
    clocks = sampler.stop()
    # the dominant force kernel's launch time: a separate pass with CUDA events
    # around every launch (direct launches, the same state continuing)
    eng.set_profiling(True)
    prof_steps = min(args.steps, 20 if args.workload == "gravity" else 200)
    eng.advance(dt, prof_steps)
    kern_ms, kern_n = eng.force_kernel_time()
    # small systems run the persistent cluster step loop: one launch per
    # chunk of steps, timed whole
    cluster = None if batch else eng.cluster_shape()
    ens = eng.ensemble_form() if batch else None
    eng.set_profiling(False)
    total_ms = max_over_ranks(float(sum(step_ms)), dist, f"cuda:{device}")
    if dist is not None:
        dist.barrier()
    value = n * args.steps * world / (total_ms / 1e3)

    # end-to-end: the drop-in right-hand side on pinned host buffers, with the
    # velocity-Verlet update on the host (SciML's loop), every step
    e2e = None
    if not args.no_e2e and not batch:
        cols = eng.cols
        pin = lambda: torch.zeros((cols, 3), dtype=torch.float64).pin_memory()
        ut, vt, at, ant = pin(), pin(), pin(), pin()
        uh, vh, ah, anh = ut.numpy(), vt.numpy(), at.numpy(), ant.numpy()
        # nbg_accel uploads v only for the thermostats whose right-hand side reads it
        v_read = wl.descs[0].thermostat in (nbg._abi.NBG_THERMO_BERENDSEN, nbg._abi.NBG_THERMO_NOSEHOOVER)
        uh[:] = u0
        vh[:] = v0
        e2e_steps = max(3, min(args.steps, 50 if args.workload == "gravity" else 200))
        eng.accel(vh, uh, out=ah)
        torch.cuda.synchronize()
        # the host loop of SciML's velocity Verlet around the drop-in: numpy
        # in-place passes over the pinned arrays (no temporaries), one
        # nbg_accel per step through the C ABI
        tmp = np.empty_like(uh)
        accel = eng.lib.nbg_accel
        ctx = eng.ctx
        p_v, p_u = nbg._abi.as_dptr(vh), nbg._abi.as_dptr(uh)
        p_a = [nbg._abi.as_dptr(ah), nbg._abi.as_dptr(anh)]
        arrs = [ah, anh]
        tarrs = [at, ant]
        hdt, hdt2 = 0.5 * dt, 0.5 * dt * dt
        # large states: torch's in-place axpy on the same pinned memory, over
        # its intra-op threads (two passes per update, as a compiled host
        # loop would make); small ones: numpy (no per-call thread start-up)
        big = uh.size >= 3 * 16384
        host_update = (f"torch add_ in place, {torch.get_num_threads()} threads" if big
                       else "numpy in place, one thread")
        t0 = time.perf_counter()
        cur = 0
        for s in range(e2e_steps):
            # u += dt v + dt^2/2 a ; a' = accel(u) ; v += dt/2 (a + a')
            if big:
                ut.add_(vt, alpha=dt).add_(tarrs[cur], alpha=hdt2)
            else:
                a_old = arrs[cur]
                np.multiply(vh, dt, out=tmp)
                np.add(uh, tmp, out=uh)
                np.multiply(a_old, hdt2, out=tmp)
                np.add(uh, tmp, out=uh)
            st = accel(ctx, p_a[cur ^ 1], p_v, p_u, 0.0)
            if st != 0:
                raise nbg.EngineError(st, "nbg_accel")
            if big:
                vt.add_(tarrs[cur], alpha=hdt).add_(tarrs[cur ^ 1], alpha=hdt)
            else:
                np.add(arrs[cur], arrs[cur ^ 1], out=tmp)
                np.multiply(tmp, hdt, out=tmp)
                np.add(vh, tmp, out=vh)
            cur ^= 1
        e2e_s = time.perf_counter() - t0
        e2e = {"value": n * e2e_steps * world / e2e_s, "unit": "atom-steps/s",
               "h2d_bytes_per_step": (2 if v_read else 1) * uh.nbytes, "d2h_bytes_per_step": ah.nbytes,
               "path": "nbg_accel (RHS drop-in) per step from pinned host buffers, velocity-Verlet update on host",
               "host_update": host_update, "steps": e2e_steps}
    elif not args.no_e2e and batch:
        # the batch's public call: nbg_run from (pageable) host buffers, state in and out
        t0 = time.perf_counter()
        ug, vg, _, _, st = eng.run(u0, v0, dt, args.steps, 0, save_trajectory=False)
        e2e_s = time.perf_counter() - t0
        e2e = {"value": n * args.steps * world / e2e_s, "unit": "atom-steps/s",
               "h2d_bytes_per_step": 2 * u0.nbytes / args.steps, "d2h_bytes_per_step": 2 * u0.nbytes / args.steps,
               "path": "nbg_run: host state uploaded, K steps, host state downloaded", "steps": args.steps}

    u_end, v_end = eng.get_state()
    traj = None
    if args.save_every > 0 and not batch:
        # run_simulation's frames (nbg_run from host buffers): saved every
        # save_every steps, against the same run without frames
        traj_steps = max(args.save_every, min(args.steps, 1000))
        eng.run(u0, v0, dt, 20, 0, save_trajectory=False)
        t0 = time.perf_counter()
        eng.run(u0, v0, dt, traj_steps, 0, save_trajectory=False)
        t_none = time.perf_counter() - t0
        t0 = time.perf_counter()
        _, _, tu, _, _ = eng.run(u0, v0, dt, traj_steps, args.save_every)
        t_frames = time.perf_counter() - t0
        traj = {"save_every": args.save_every, "steps": traj_steps, "frames": len(tu),
                "us_per_step": 1e6 * t_frames / traj_steps, "us_per_step_no_frames": 1e6 * t_none / traj_steps,
                "path": "nbg_run from host buffers, positions and velocities saved (run_simulation)"}
    work, unit, bound = algorithmic_work(args.workload, n, eng)
    avg_kern = kern_ms / max(kern_n, 1)
    if cluster is not None or ens is not None:
        avg_kern = kern_ms / prof_steps  # per step of the multi-step launches
    achieved = work / (avg_kern / 1e3) / (1e12 if unit == "TFLOP/s" else 1e9)
    peaks = measured_peaks()
    if unit == "TFLOP/s":
        peak = peak_fp32
        peak_src = "FP32 FMA probe measured in this run (nbg_probe_fp32_peak)"
    else:
        peak = peaks.get("hbm_gbs", 6800.0)
        peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    kernel_name = ("k_gravity" if args.workload == "gravity" else "k_cluster_vv" if cluster else
                   "k_ensemble" if ens else "k_force_list")
    form = eng.force_form() if kernel_name == "k_force_list" else None
    if form is not None and form[1]:
        # the fixed-point kernel: per-warp list staging up to 16 lanes per atom
        kernel_name = "k_force_fxw" if form[0] <= 16 and not os.environ.get("NBG_FX_BLOCK") else "k_force_fx"
    traffic = profile_traffic(f"{kernel_name}:{w['name']}")
    roofline = {"bound": bound, "achieved": achieved, "peak": peak, "unit": unit,
                "frac": (achieved / peak) if peak else None, "traffic": traffic, "kernel": kernel_name,
                "kernel_ms": avg_kern, "kernel_launches": kern_n, "peak_source": peak_src}
    if cluster is not None:
        # a few kB per step stay on chip: the bound is the issue rate of the
        # cluster's SMs (4 warp instructions per clock each) for the step's
        # warp instructions (ncu), at the sampled SM clock
        inst = profile_value(f"k_cluster_vv:{w['name']}", "issue.json")
        mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz") or 2070.0
        floor_us = inst / (cluster[0] * 4 * mhz) if inst else None
        step_us = 1e3 * avg_kern
        roofline.update(bound="issue", achieved=step_us, peak=floor_us, unit="us/step",
                        frac=(floor_us / step_us) if floor_us else None,
                        peak_source=(f"issue floor: {inst} warp instructions per step (ncu) / "
                                     f"({cluster[0]} SMs x 4 per clock x {mhz:.0f} MHz)"),
                        algorithmic_bytes_per_step=work, hbm_frac=achieved / peak if peak else None)
        roofline["kernel_ms_is"] = f"per step: {prof_steps} steps in {kern_n} launch(es) of the whole step loop"
        roofline["cluster"] = {"ctas": cluster[0], "lanes_per_atom": cluster[1]}
        # the per-call floor: an empty kernel of the same launch shape (after the timed region)
        lf = eng.cluster_launch_floor()
        if lf is not None:
            roofline["launch_floor_us"] = {"one_at_a_time": lf[0], "back_to_back": lf[1]}
    if ens is not None:
        # the whole step of every replica in one launch: bound by instruction
        # issue and latency (positions in shared memory, FP64 integration),
        # not by DRAM: the floor is the step's warp instructions (ncu) over
        # all SMs at 4 per clock; the HBM fraction of the 334 B per atom-step
        # of algorithmic traffic is kept beside it
        inst = profile_value(f"k_ensemble:{w['name']}", "issue.json")
        mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz") or 2070.0
        sms = torch.cuda.get_device_properties(device).multi_processor_count
        floor_ms = inst / (sms * 4 * mhz * 1e3) if inst else None
        roofline.update(bound="issue", achieved=avg_kern, peak=floor_ms, unit="ms/step",
                        frac=(floor_ms / avg_kern) if floor_ms else None,
                        peak_source=(f"issue floor: {inst} warp instructions per step (ncu) / "
                                     f"({sms} SMs x 4 per clock x {mhz:.0f} MHz)"),
                        algorithmic_bytes_per_step=work, hbm_frac=achieved / peak if peak else None)
        roofline["kernel_ms_is"] = (f"per step: {prof_steps} steps in {kern_n} launch(es) of the whole step loop "
                                    "(a CTA per replica)")
    config = {"workload": w["name"], "N": n, "dt": dt, "integrator": "velocity Verlet",
              "l2": ("512 MB buffer written between timed steps (L2 flushed)" if flush_steps else
                     "working set larger than L2" if batch else "no flush (state L2-resident across steps)"),
              "parallelism": "replicas only" if world > 1 else "single GPU"}
    if args.workload == "gravity":
        config["gravity_precision"] = "plain FP32 positions" if args.grav_plain else "hi/lo split positions (compensated)"
    else:
        if args.workload == "water":
            config["spcfw"] = SPCFW_CONFIG
        d0 = wl.descs[0]
        re = int(d0.rebuild_every)
        config["verlet_list"] = {"skin": float(d0.skin),
                                 "rebuild": (f"every {re} steps and " if re > 0 else "") +
                                            "whenever an atom moved more than skin/2 since the last build"}
    if tuned is not None:
        config["lanes_per_atom"] = tuned[0]
        config["autotune_force_ms"] = tuned[1]
    if batch:
        config.update(integrator="BAOAB Langevin (gamma=1)", replicas=len(wl.sizes),
                      atoms_min=int(min(wl.sizes)), atoms_max=int(max(wl.sizes)))
        config["step_loop"] = ("persistent: one launch per chunk of steps, a CTA per replica" if ens else
                               "CUDA graphs of per-step kernels")
    if ens_tuned is not None:
        form, ms = ens_tuned
        config["ensemble_form"] = (
            {"lanes_per_atom": form[0], "threads_per_replica": form[1],
             "cells": "list radius, 3x3x3" if form[2] == 1 else "half list radius, 5x5x5"} if form is not None
            else "per-step kernels in CUDA graphs (faster than every loop form in the tuner)")
        config["ensemble_autotune"] = {
            "ms_per_step_loop_forms": [round(float(x), 4) for x in ms[:12]],
            "ms_per_step_step_graphs": round(float(ms[12]), 4),
            "window": f"{ENS_TUNE_STEPS} steps from the state after {ENS_TUNE_AFTER} untimed steps, "
                      "each form from the same state with a full list build at its first step"}
    line = {"metric": "atom-steps/s", "value": value, "unit": "atom-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 pair forces, f64 state" + ("+bonded" if args.workload == "water" else ""),
            "data": "synthetic (seeded generator, no dataset)", "config": config,
            "roofline": roofline, "e2e": e2e, "gpu_launches": launches, "clocks": clocks}
    if traj is not None:
        line["trajectory"] = traj
    if not batch:
        e_end = eng.energy(u_end, v_end)
        drift_key = "gravity" if args.workload == "gravity" else "potential"
        E0 = e_start["kinetic"] + e_start[drift_key]
        E1 = e_end["kinetic"] + e_end[drift_key]
        if args.workload == "water":
            # Berendsen at 300 K from a jittered lattice: the thermostat removes
            # the energy the melting lattice releases, so energy is not conserved
            line["energy_change_rel_thermostatted"] = (E1 - E0) / abs(E0) if E0 else None
        else:
            line["energy_drift_rel"] = (E1 - E0) / abs(E0) if E0 else None
        if args.workload != "gravity":
            line["temperature_start"] = e_start["temperature"]
            line["temperature_end"] = e_end["temperature"]
    else:
        offs = np.concatenate([[0], np.cumsum(wl.sizes)])
        T_end = [float((v_end[offs[r]:offs[r + 1]] ** 2).sum() / (3 * wl.sizes[r])) for r in range(len(wl.sizes))]
        T_tgt = [float(d.thermo_T) for d in wl.descs]
        line["temperature_rel_err_mean"] = float(np.mean(np.abs(np.array(T_end) / np.array(T_tgt) - 1)))
    if args.workload == "water":
        line["ns_per_day"] = (1e3 / (total_ms / args.steps)) * dt * 1e-3 * 86400
    if rank == 0 and world == 1 and not args.no_cpu:
        oracle = G.load_oracle()
        line["cpu_baseline"] = cpu_baseline(oracle, wl)
        if args.workload in ("gravity", "lj"):
            # force accuracy on atoms 0..255 of the end state (a thermalised
            # liquid: on the starting lattice the LJ forces cancel to ~0)
            ns = min(256, n)
            a_ref = oracle.partial_accel(wl.descs[0], u_end, 0, ns)
            eng.set_state(u_end, v_end)
            eng.compute_forces()
            a_gpu = eng.get_accel()[:ns]
            line["force_rel_rmse"] = float(np.linalg.norm(a_gpu - a_ref) / np.linalg.norm(a_ref))
            if args.workload == "gravity" and not args.grav_plain:
                # the same steps with plain FP32 position differences everywhere
                dp = wl.descs[0]
                dp.flags |= nbg._abi.NBG_FLAG_GRAV_PLAIN
                ep = nbg.Engine([dp], device)
                ep.set_stream(stream.cuda_stream)
                ep.set_state(u0, v0)
                ep.advance(dt, args.warmup)
                torch.cuda.synchronize()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                ep.advance(dt, args.steps)
                e1.record(stream)
                torch.cuda.synchronize()
                ms_plain = e0.elapsed_time(e1) / args.steps
                ep.set_state(u_end, v_end)
                ep.compute_forces()
                a_plain = ep.get_accel()[:ns]
                line["plain_fp32_positions"] = {
                    "value": n / (ms_plain / 1e3), "unit": "atom-steps/s", "ms_per_step": ms_plain,
                    "l2": "no flush (steps back to back)",
                    "force_rel_rmse": float(np.linalg.norm(a_plain - a_ref) / np.linalg.norm(a_ref))}
                ep.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
