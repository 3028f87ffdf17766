"""Host-side mirror of the reference API: constructors, show strings,
marshalling of the system descriptor, and the C ABI's exported symbols.
CPU only (no kernel is called)."""
import ctypes
import math
import os
import re

import numpy as np
import pytest

import systems as S

nbg = S.nbg
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_parameter_defaults_and_show():
    """lennard_jones_test.jl:152-166, electrostatics_test.jl:70-82, gravitational_test.jl:283-292."""
    p = nbg.LennardJonesParameters()
    assert (p.eps, p.sigma, p.R, p.sigma2, p.R2) == (1.0, 1.0, 2.5, 1.0, 6.25)
    assert p.show() == "Lennard-Jones:\n\tϵ:1.0\n\tσ:1.0\n\tR:2.5\n"
    assert nbg.LennardJonesParameters(2, 5, 10).show() == "Lennard-Jones:\n\tϵ:2\n\tσ:5\n\tR:10\n"
    assert nbg.ElectrostaticParameters().k == 9.0e9
    assert nbg.ElectrostaticParameters(9e9, 8.0).R2 == 64.0
    assert nbg.ElectrostaticParameters().show() == "Electrostatic:\n\tk:9.0e9\n"
    assert nbg.ElectrostaticParameters(1.0).show() == "Electrostatic:\n\tk:1.0\n"
    assert nbg.GravitationalParameters().G == 6.67408e-11
    assert nbg.GravitationalParameters().show() == "Gravitational:\n\tG:6.67408e-11\n"
    assert nbg.GravitationalParameters(35.67).show() == "Gravitational:\n\tG:35.67\n"


def test_potential_system_show():
    """custom_potential_body.jl:49-59."""
    p1 = nbg.MassBody((1, 0, 0), (0, 0, 0), 1.0)
    p2 = nbg.MassBody((-1, 0, 0), (0, 0, 0), 1.0)
    s = nbg.PotentialNBodySystem([p1, p2], [":lennard_jones", ":electrostatic", ":gravitational", ":magnetostatic"])
    assert s.show() == ("Potentials: \nLennard-Jones:\n\tϵ:1.0\n\tσ:1.0\n\tR:2.5\nElectrostatic:\n\tk:9.0e9\n"
                        "Magnetostatic:\n\tμ/4π:1.0e-7\nGravitational:\n\tG:6.67408e-11\n")


def test_simulation_show():
    """lennard_jones_test.jl:37-41."""
    sim, _ = S.lj_two_body()
    assert sim.system.show() == "Potentials: \nLennard-Jones:\n\tϵ:1.0\n\tσ:1.0\n\tR:Inf\n"
    assert sim.show() == ("Timespan: (0.0, 1.0)\nBoundary conditions: InfiniteBox{Float64}([-Inf, Inf, -Inf, Inf, "
                          "-Inf, Inf])\nPotentials: \nLennard-Jones:\n\tϵ:1.0\n\tσ:1.0\n\tR:Inf\n")


def test_periodic_boundary_indexing():
    """lennard_jones_test.jl:168-179."""
    pbc = nbg.PeriodicBoundaryConditions(15.0e-6)
    boundary = [0.0, 15.0e-6, 0.0, 15.0e-6, 0.0, 15.0e-6]
    for i in range(1, 7):
        assert boundary[i - 1] == pbc[i]


def test_water_thermostat_data():
    """water_test.jl:95-134: n = 6, nc = 4, Nose-Hoover index 19 (1-based)."""
    L, lj, el, spc, mH2O = S.water_params()
    b = [nbg.MassBody((L / 3, L / 3, 2 * L / 3), (0, 0, 0), mH2O), nbg.MassBody((L / 3, 2 * L / 3, L / 3), (0, 0, 0), mH2O)]
    w = S.WATER
    water = nbg.WaterSPCFw(b, w["mH"], w["mO"], w["qH"], w["qO"], lj, el, spc)
    n, nc, ndf = nbg.get_degrees_of_freedom(water)
    assert (n, nc) == (6, 4)
    assert len(nbg.get_masses(water)) == n
    sim = nbg.NBodySimulation(water, (0.0, 1.0), nbg.CubicPeriodicBoundaryConditions(L),
                              nbg.NoseHooverThermostat(275, 0.1), S.KB_KJ)
    u0, v0, _ = nbg.gather_bodies_initial_coordinates(sim)
    assert u0.shape == (7, 3)
    assert 3 * n + 1 == 19  # zeta at the first row of the extra column
    desc, keep = nbg.system_descriptor(sim)
    assert desc.n == 6 and desc.thermostat == nbg._abi.NBG_THERMO_NOSEHOOVER


def test_water_hydrogen_placement():
    """nbody_to_ode.jl:37-55: H1 = O + (rOH,0,0), H2 = O + (cos a rOH, 0, sin a rOH)."""
    L, lj, el, spc, mH2O = S.water_params()
    w = S.WATER
    water = nbg.WaterSPCFw([nbg.MassBody((1, 2, 3), (0.1, 0, 0), mH2O)], w["mH"], w["mO"], w["qH"], w["qO"], lj, el, spc)
    sim = nbg.NBodySimulation(water, (0.0, 1.0), nbg.CubicPeriodicBoundaryConditions(L), S.KB_KJ)
    u0, v0, _ = nbg.gather_bodies_initial_coordinates(sim)
    assert np.allclose(u0[1], [1 + w["rOH"], 2, 3])
    assert np.allclose(u0[2], [1 + math.cos(w["aHOH"]) * w["rOH"], 2, 3 + math.sin(w["aHOH"]) * w["rOH"]])
    assert np.all(v0 == [0.1, 0, 0])


def test_custom_potential_rejected():
    """A Julia-side custom potential (test/shared/custom_potential_body.jl)
    has no GPU kernel: the engine refuses it instead of computing on the CPU."""
    class Custom(nbg.PotentialParameters):
        pass
    s = nbg.PotentialNBodySystem([nbg.MassBody((0, 0, 0), (0, 0, 0), 1.0)], {"custom_potential_params": Custom()})
    sim = nbg.NBodySimulation(s, (0.0, 1.0))
    with pytest.raises(nbg.EngineError):
        nbg.system_descriptor(sim)


def test_descriptor_layout_matches_header():
    """The ctypes struct has the layout gcc gives the C struct of include/nbg.h."""
    src = r'''
    #include <stddef.h>
    #include <stdio.h>
    #include "nbg.h"
    int main(void) {
      printf("%zu %zu %zu %zu %zu %zu\n", sizeof(nbg_system_desc), offsetof(nbg_system_desc, box),
             offsetof(nbg_system_desc, seed), offsetof(nbg_system_desc, flags), sizeof(nbg_energies),
             sizeof(nbg_run_stats));
      return 0; }
    '''
    import subprocess
    import tempfile
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        open(c, "w").write(src)
        exe = os.path.join(d, "t")
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        vals = [int(x) for x in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()]
    A = nbg._abi
    assert vals == [ctypes.sizeof(A.NbgSystemDesc), A.NbgSystemDesc.box.offset, A.NbgSystemDesc.seed.offset,
                    A.NbgSystemDesc.flags.offset, ctypes.sizeof(A.NbgEnergies), ctypes.sizeof(A.NbgRunStats)]


def _header_functions():
    text = open(os.path.join(ROOT, "include", "nbg.h")).read()
    return sorted(set(re.findall(r"NBG_API[^;(]*?\b(nbg_\w+)\s*\(", text)))


def test_library_exports_every_header_symbol():
    """libnbg.so (built for sm_103a) loads without a GPU and exports every
    function include/nbg.h declares; the ctypes table covers them all."""
    import __graft_entry__ as g
    lib_build = g._load_by_path("nbg_lib_build", os.path.join(ROOT, "nbodysimulator.jl_gb300", "build.py"))
    path = lib_build.build()
    lib = ctypes.CDLL(path)
    names = _header_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(nbg._abi.SIGNATURES), set(names) ^ set(nbg._abi.SIGNATURES)
    loaded = nbg.load_library()
    assert loaded.nbg_abi_version() == nbg._abi.NBG_ABI_VERSION
    assert b"sm_103a" in loaded.nbg_version()


def test_debug_library_builds_and_exports_every_header_symbol():
    """The debug build (nvcc -DNBG_DEBUG: index checks on every neighbour and
    cell table read) compiles for sm_103a, loads without a GPU and exports the
    same functions; NBG_ERR_INDEX is in the header and in the status names."""
    import __graft_entry__ as g
    lib_build = g._load_by_path("nbg_lib_build", os.path.join(ROOT, "nbodysimulator.jl_gb300", "build.py"))
    path = lib_build.build(debug=True)
    assert path.endswith("libnbg_debug.so")
    lib = ctypes.CDLL(path)
    for n in _header_functions():
        assert hasattr(lib, n), n
    assert lib.nbg_abi_version() == nbg._abi.NBG_ABI_VERSION
    with open(os.path.join(ROOT, "include", "nbg.h")) as f:
        assert re.search(r"NBG_ERR_INDEX\s*=\s*-9", f.read())
    assert nbg._abi.STATUS_NAMES[-9] == "NBG_ERR_INDEX"


def test_result_analysis_at_saved_times():
    """gravitational_test.jl:26-41: get_position / get_velocity of body 1 at
    the first saved time are its initial values exactly, get_masses the
    bodies' masses; and electrostatics_test.jl:31-39: the charges and masses
    the descriptor carries (obtain_data_for_electrostatic_interaction). The
    result here is hand-made, so no kernel runs."""
    sim = S.figure8()
    u0, v0 = S.state(sim)
    res = nbg.SimulationResult(nbg.simulation.Solution([0.0, 1.0], [u0, u0 + 0.5], [v0, v0 - 0.5], 1), sim)
    r1 = nbg.get_position(res, 0.0, 1)
    v1 = nbg.get_velocity(res, 0.0, 1)
    for i, (r, v) in enumerate(zip((-0.995492, 0.0, 0.0), (-0.347902, -0.53393, 0.0))):
        assert r1[i] == r and v1[i] == v
    assert list(nbg.get_masses(sim.system)) == [1.0, 1.0, 1.0]
    assert np.array_equal(nbg.get_position(res, 1.0, 2), u0[1] + 0.5)
    assert np.array_equal(nbg.get_position(res, 1.0), (u0 + 0.5).T)

    k, q1, q2, m1, m2 = 9.0e9, 1.0e-3, -1.0e-3, 100.0, 0.1
    p1 = nbg.ChargedParticle((0.0, 0.0, 0.0), (0.0, 0.0, 0.0), m1, q1)
    p2 = nbg.ChargedParticle((100.0, 0.0, 0.0), (0.0, 1.0, 0.0), m2, q2)
    sim = nbg.NBodySimulation(nbg.ChargedParticles([p1, p2], k), (0.0, 1.0))
    desc, keep = nbg.system_descriptor(sim)
    qs = np.ctypeslib.as_array(desc.charge, shape=(2,))
    ms = np.ctypeslib.as_array(desc.mass, shape=(2,))
    assert qs[0] == q1 and qs[1] == q2
    assert ms[0] == m1 and ms[1] == m2
    assert desc.el_k == k


def test_rdf_histogram_argument_checks():
    """nbg_rdf_histogram refuses bad arguments before any device work
    (NBG_ERR_ARG = -1): bin counts outside 1..16384, a column outside the
    frame, a non-positive or non-finite box, missing buffers."""
    lib = nbg.load_library()
    frames = np.zeros((2, 10, 3))
    hist = np.zeros(16385)
    idx = np.arange(10, dtype=np.int32)
    ip = idx.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))

    def call(idx_p=ip, nidx=10, L=2.0, maxbin=100, fr=frames.ctypes.data, out=hist.ctypes.data):
        return lib.nbg_rdf_histogram(fr, 2, 10, idx_p, nidx, L, maxbin, 0, out)

    assert call(maxbin=0) == -1
    assert call(maxbin=16385) == -1
    assert call(L=0.0) == -1 and call(L=-1.0) == -1 and call(L=float("inf")) == -1
    bad = np.array([0, 10], dtype=np.int32)
    assert call(idx_p=bad.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), nidx=2) == -1
    neg = np.array([-1], dtype=np.int32)
    assert call(idx_p=neg.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), nidx=1) == -1
    assert call(out=None) == -1
    assert call(fr=None) == -1
    assert call(idx_p=None) == -1
    assert lib.nbg_rdf_kernel_times(None) == -1


def test_element_types():
    """interface_test.jl: the reference runs BigFloat and Float32 problems.
    Here float32 input is accepted and computed in float64; arbitrary
    precision (Decimal, Fraction, numpy longdouble standing in for BigFloat)
    has no GPU kernel and the descriptor builder refuses it with
    NBG_ERR_UNSUPPORTED (-6), so the caller keeps it on the CPU."""
    from decimal import Decimal
    from fractions import Fraction

    f32 = np.float32
    b1 = nbg.MassBody(np.array([1, 0, 0], dtype=f32), np.array([0, 0.5, 0], dtype=f32), f32(1))
    b2 = nbg.MassBody(np.array([-1, 0, 0], dtype=f32), np.array([0, -0.5, 0], dtype=f32), f32(1))
    sim = nbg.NBodySimulation(nbg.GravitationalSystem([b1, b2], f32(1)), (f32(0), f32(1)), nbg.InfiniteBox(),
                              f32(1.38e-23))
    desc, keep = nbg.system_descriptor(sim)
    assert desc.n == 2 and desc.grav_G == 1.0

    def refused(make):
        with pytest.raises(nbg.EngineError) as e:
            nbg.system_descriptor(make())
        assert e.value.status == -6

    big = lambda x: Decimal(str(x))
    refused(lambda: nbg.NBodySimulation(
        nbg.GravitationalSystem([nbg.MassBody((big(1), big(0), big(0)), (big(0), big(0.5), big(0)), big(1)),
                                 nbg.MassBody((big(-1), big(0), big(0)), (big(0), big(-0.5), big(0)), big(1))],
                                big(1)), (0.0, 1.0)))
    p0 = nbg.MassBody((0, 0, 0), (0, 0, 0), 1.0)
    p1 = nbg.MassBody((2, 0, 0), (0, 0, 0), 1.0)
    refused(lambda: nbg.NBodySimulation(nbg.PotentialNBodySystem(
        [p0, p1], {"lennard_jones": nbg.LennardJonesParameters(big(1), big(1), big(2.5))}), (0.0, 0.1)))
    refused(lambda: nbg.NBodySimulation(nbg.GravitationalSystem([p0, p1], 1.0), (Fraction(0), Fraction(1, 10))))
    if np.dtype(np.longdouble).itemsize > 8:
        ld = np.longdouble
        refused(lambda: nbg.NBodySimulation(nbg.GravitationalSystem(
            [nbg.MassBody(np.array([1, 0, 0], dtype=ld), (0, 0, 0), 1.0), p1], 1.0), (0.0, 1.0)))
