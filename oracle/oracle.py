"""ctypes wrapper of the FP64 oracle (oracle.c).

TEST INFRASTRUCTURE ONLY: the oracle the CUDA engine is tested against. Only tests/, the
smoke check and bench.py's CPU-baseline leg may import this module. It takes
the same nbg_system_desc the engine takes (built by the package's
system_descriptor), so both sides see identical inputs.
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import build as _build  # noqa: E402

_lib = None
_dp = ctypes.POINTER(ctypes.c_double)


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        _lib = ctypes.CDLL(path)
        _lib.oracle_accel.argtypes = [ctypes.c_void_p, _dp, _dp, _dp, ctypes.c_double]
        _lib.oracle_run.restype = ctypes.c_int64
        _lib.oracle_run.argtypes = [ctypes.c_void_p, _dp, _dp, ctypes.c_double, ctypes.c_int64, ctypes.c_int64,
                                    _dp, _dp]
        _lib.oracle_energy.argtypes = [ctypes.c_void_p, _dp, _dp, ctypes.c_void_p]
        _lib.oracle_pair_list.restype = ctypes.c_int64
        _lib.oracle_pair_list.argtypes = [ctypes.c_void_p, _dp, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32),
                                          ctypes.c_int64]
        _lib.oracle_partial_accel.argtypes = [ctypes.c_void_p, _dp, _dp, ctypes.c_int64, ctypes.c_int64]
        _lib.oracle_set_threads.argtypes = [ctypes.c_int]
        _lib.oracle_md_temperature.restype = ctypes.c_double
        _lib.oracle_md_temperature.argtypes = [_dp, _dp, ctypes.c_double, ctypes.c_int64, ctypes.c_int64]
        _lib.oracle_uniform.restype = ctypes.c_double
        _lib.oracle_uniform.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64]
        _lib.oracle_normals3.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64, _dp]
        _lib.oracle_rdf_histogram.argtypes = [_dp, ctypes.c_int64, ctypes.c_int64, ctypes.POINTER(ctypes.c_int32),
                                              ctypes.c_int64, ctypes.c_double, ctypes.c_int32, _dp]
    return _lib


def _p(a):
    return a.ctypes.data_as(_dp)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64).copy()


def set_threads(n):
    lib().oracle_set_threads(int(n))


def accel(desc, v, u, t=0.0):
    """soode_system!(dv, v, u, p, t); returns (dv, v) (v may be modified by
    the Nose-Hoover term)."""
    u = _f64(u)
    v = _f64(v)
    dv = np.zeros_like(u)
    lib().oracle_accel(ctypes.byref(desc), _p(dv), _p(v), _p(u), float(t))
    return dv, v


def run(desc, u, v, dt, nsteps, save_every=0, trajectory=False):
    """Returns (u, v) after nsteps, or (u, v, traj_u, traj_v) with trajectory."""
    u = _f64(u)
    v = _f64(v)
    tu = tv = None
    if trajectory:
        nframes = (nsteps // save_every + 2) if save_every > 0 else 2
        tu = np.zeros((nframes,) + u.shape)
        tv = np.zeros((nframes,) + u.shape)
    frames = lib().oracle_run(ctypes.byref(desc), _p(u), _p(v), float(dt), int(nsteps), int(save_every),
                              _p(tu) if tu is not None else None, _p(tv) if tv is not None else None)
    if trajectory:
        return u, v, tu[:frames], tv[:frames]
    return u, v


class _Energies(ctypes.Structure):
    _fields_ = [(k, ctypes.c_double) for k in (
        "kinetic", "lennard_jones", "electrostatic", "bonds", "angles", "gravity",
        "potential", "total", "temperature")]


def energy(desc, u, v):
    out = _Energies()
    u = _f64(u)
    v = _f64(v)
    lib().oracle_energy(ctypes.byref(desc), _p(u), _p(v), ctypes.byref(out))
    return {k: getattr(out, k) for k, _ in out._fields_}


def pair_list(desc, u, which):
    u = _f64(u)
    cnt = lib().oracle_pair_list(ctypes.byref(desc), _p(u), int(which), None, 0)
    pairs = np.zeros((max(cnt, 1), 2), dtype=np.int32)
    lib().oracle_pair_list(ctypes.byref(desc), _p(u), int(which),
                           pairs.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), cnt)
    return pairs[:cnt]


def partial_accel(desc, u, i0, i1):
    u = _f64(u)
    dv = np.zeros((i1 - i0, 3))
    lib().oracle_partial_accel(ctypes.byref(desc), _p(u), _p(dv), int(i0), int(i1))
    return dv


def uniform(seed, atom, step):
    return lib().oracle_uniform(seed, atom, step)


def normals3(seed, atom, step):
    out = np.zeros(3)
    lib().oracle_normals3(seed, atom, step, _p(out))
    return out


def rdf_histogram(frames, idx, L, maxbin=1000):
    """rdf's histogram (nbody_simulation_result.jl:664-709) over frames of
    shape (nframes, ncols, 3) for the atoms idx; float64 counts."""
    frames = np.ascontiguousarray(frames, dtype=np.float64)
    idx = np.ascontiguousarray(idx, dtype=np.int32)
    hist = np.zeros(maxbin)
    lib().oracle_rdf_histogram(_p(frames), frames.shape[0], frames.shape[1],
                               idx.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), len(idx), float(L),
                               int(maxbin), _p(hist))
    return hist
