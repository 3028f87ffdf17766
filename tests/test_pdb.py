"""PDB trajectories (nbody_simulation_result.jl:786-1001): the writer's
records and columns, and the reader against the reference's own fixture and
known answers (test/water_test.jl:155-248, test/lennard_jones_test.jl:99-117).
Host-side text I/O: these run on the CPU with hand-made SimulationResults."""
import io
import math
import os

import numpy as np

import systems as S

nbg = S.nbg
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _result(sim, ts, frames):
    u = [np.asarray(f, dtype=np.float64) for f in frames]
    return nbg.SimulationResult(nbg.simulation.Solution(ts, u, [np.zeros_like(x) for x in u], len(ts) - 1), sim)


def _water_sim(pos, L):
    bodies = nbg.workloads.water_molecules(pos, np.zeros_like(pos))
    lj = nbg.LennardJonesParameters(0.650299, 0.3165492, 0.9)
    el = nbg.ElectrostaticParameters(nbg.workloads.K_EL, 0.9)
    spc = nbg.SPCFwParameters(0.1012, 113.24 * math.pi / 180, nbg.workloads.SPCFW_KB, nbg.workloads.SPCFW_KA)
    water = nbg.WaterSPCFw(bodies, nbg.workloads.M_H, nbg.workloads.M_O, 0.41, -0.82, lj, el, spc)
    return nbg.NBodySimulation(water, (0.0, 1.0), nbg.CubicPeriodicBoundaryConditions(L), S.KB_KJ)


def _counts(text):
    steps = sum(1 for s in text.split("\n") if len(s) >= 10 and s[:10] == "REMARK 250")
    atoms = sum(1 for s in text.split("\n") if len(s) >= 6 and s[:6] == "HETATM")
    return steps, atoms


def test_pdb_lj_records():
    """lennard_jones_test.jl:99-117: one REMARK 250 per saved time and one
    HETATM per body in each."""
    L = 5 * 0.34
    bodies = nbg.generate_bodies_in_cell_nodes(27, 39.95, 0.1, L, rng=np.random.default_rng(0))
    sim = nbg.NBodySimulation(nbg.PotentialNBodySystem(bodies, {"lennard_jones": nbg.LennardJonesParameters()}),
                              (0.0, 1.0), nbg.CubicPeriodicBoundaryConditions(L), 1.0)
    u0 = np.array([b.r for b in bodies])
    res = _result(sim, [0.0, 0.5, 1.0], [u0, u0 + 0.01, u0 - 0.02])
    text = io.StringIO()
    nbg.write_pdb_data(text, res)
    steps, atoms = _counts(text.getvalue())
    assert steps == len(res.solution.t) and atoms / steps == len(bodies)


def test_pdb_water_records():
    """water_test.jl:155-190: HETATM / timesteps / 3 = molecules."""
    pos, _, L = nbg.workloads.spcfw_water_box(2, seed=1)
    res = _result(_water_sim(pos, L), [0.0, 0.0005, 0.001], [pos, pos + 0.001, pos - 0.001])
    text = io.StringIO()
    nbg.write_pdb_data(text, res)
    steps, atoms = _counts(text.getvalue())
    assert steps == 3 and atoms / steps / 3 == 2


def test_pdb_columns():
    """The reference's columns, worked by hand: angstrom, wrapped into the
    box (x - L floor(x / L)), H sites at the wrapped O plus their offsets,
    Julia's printing of the time."""
    bodies = [nbg.MassBody((1.23456, -0.5, 12.0), (0, 0, 0), 1.0), nbg.MassBody((3.0, 4.0, 5.0), (0, 0, 0), 1.0)]
    sim = nbg.NBodySimulation(nbg.PotentialNBodySystem(bodies, {"lennard_jones": nbg.LennardJonesParameters()}),
                              (0.0, 1.0), nbg.CubicPeriodicBoundaryConditions(10.0), 1.0)
    u0 = np.array([b.r for b in bodies])
    res = _result(sim, [0.0, 1e-5], [u0, u0])
    text = io.StringIO()
    nbg.write_pdb_data(text, res)
    lines = text.getvalue().split("\n")
    assert lines[0] == "MODEL     1"
    assert lines[1] == "REMARK 250 time=0.0 steps"
    assert lines[2] == "HETATM    1  Ar  Ar     1      12.346  95.000  20.000  1.00  0.00          Ar"
    assert lines[3] == "HETATM    2  Ar  Ar     2      30.000  40.000  50.000  1.00  0.00          Ar"
    assert lines[4] == "ENDMDL"
    assert lines[5] == "MODEL     2" and lines[6] == "REMARK 250 time=1.0e-5 steps"
    assert lines[-1] == "" and lines[-2] == "ENDMDL"

    pos = np.array([[1.05, 0.2, -0.01], [1.15, 0.2, -0.01], [1.02, 0.29, -0.01]])
    res = _result(_water_sim(pos, 1.0), [0.0005], [pos])
    text = io.StringIO()
    nbg.write_pdb_data(text, res)
    lines = text.getvalue().split("\n")
    assert lines[:6] == [
        "MODEL     1",
        "REMARK 250 time=0.0005 picoseconds",
        "HETATM    1  O   HOH     1       0.500   2.000   9.900  1.00  0.00           O",
        "HETATM    2  H1  HOH     1       1.500   2.000   9.900  1.00  0.00           H",
        "HETATM    3  H2  HOH     1       0.200   2.900   9.900  1.00  0.00           H",
        "ENDMDL",
    ]


def test_extract_from_pdb_reference_fixture():
    """water_test.jl:192-248: the reference's two-model, three-molecule text
    (tests/golden/water3_two_frames.pdb, written by make_pdb_fixture.py from
    the reference test) and its known answers: positions of the first model in
    nm to 5e-5, velocities zero."""
    with open(os.path.join(GOLDEN, "water3_two_frames.pdb")) as f:
        bodies = nbg.extract_from_pdb(f)
    assert len(bodies) == 3
    eps = 0.00005
    assert abs(bodies[0].O.r[0] - 1.8642) <= eps and abs(bodies[0].O.r[1] - 1.8642) <= eps
    assert abs(bodies[0].O.r[2] - 0.0) <= eps
    assert abs(bodies[1].H1.r[0] - 0.0957) <= eps and abs(bodies[1].H1.r[1]) <= eps
    assert abs(bodies[1].H1.r[2] - 0.3107) <= eps
    assert abs(bodies[2].H2.r[0] - 1.8882) <= eps and abs(bodies[2].H2.r[1] - 1.7715) <= eps
    assert abs(bodies[2].H2.r[2] - 0.6214) <= eps
    assert all(abs(c) <= eps for c in bodies[2].H2.v)
    assert bodies[0].O.m == 15.999 and bodies[0].H1.m == 1.00794
    # the loaded molecules build a water system, as the reference test does
    water = nbg.WaterSPCFw(bodies, nbg.workloads.M_H, nbg.workloads.M_O, 0.41, -0.82,
                           nbg.LennardJonesParameters(0.650299, 0.3165492, 0.9),
                           nbg.ElectrostaticParameters(nbg.workloads.K_EL, 0.9),
                           nbg.SPCFwParameters(0.1012, 113.24 * math.pi / 180, nbg.workloads.SPCFW_KB,
                                               nbg.workloads.SPCFW_KA))
    assert len(water.bodies) == 3


def test_pdb_round_trip(tmp_path):
    """save_to_pdb then load_water_molecules_from_pdb: the first frame's
    whole-molecule wrapped positions, to the 1e-3 angstrom of the columns."""
    pos, _, L = nbg.workloads.spcfw_water_box(64, seed=3)
    rng = np.random.default_rng(4)
    f0 = pos + rng.normal(scale=0.5, size=pos.shape)  # some sites outside the box
    res = _result(_water_sim(pos, L), [0.0, 0.0005], [f0, f0 + 0.001])
    path = str(tmp_path / "w.pdb")
    nbg.save_to_pdb(res, path)
    mols = nbg.load_water_molecules_from_pdb(path)
    assert len(mols) == 64
    got = np.array([[m.O.r, m.H1.r, m.H2.r] for m in mols]).reshape(-1, 3)
    cc0 = 10 * f0.T
    cc = cc0 - 10 * L * np.floor(cc0 / (10 * L))
    cc[:, 1::3] = (cc[:, 0::3] + cc0[:, 1::3]) - cc0[:, 0::3]
    cc[:, 2::3] = (cc[:, 0::3] + cc0[:, 2::3]) - cc0[:, 0::3]
    assert np.abs(got - cc.T / 10).max() <= 0.5e-4 + 1e-12
