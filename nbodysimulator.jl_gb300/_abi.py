"""ctypes view of the C ABI declared in include/nbg.h (libnbg.so).

The library is the only compute path of this package: if it is missing or
fails to load, every entry point raises instead of falling back to the CPU.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# NBG_DEBUG=1 selects the debug build (libnbg_debug.so: bounds checks on every
# neighbour and cell index a kernel reads, reported as NBG_ERR_INDEX)
LIB_PATH = os.path.join(HERE, "libnbg_debug.so" if os.environ.get("NBG_DEBUG") == "1" else "libnbg.so")

NBG_ABI_VERSION = 1

NBG_OK = 0
STATUS_NAMES = {
    -1: "NBG_ERR_ARG",
    -2: "NBG_ERR_CUDA",
    -3: "NBG_ERR_CAPACITY",
    -4: "NBG_ERR_NONFINITE",
    -5: "NBG_ERR_TIMEOUT",
    -6: "NBG_ERR_UNSUPPORTED",
    -7: "NBG_ERR_RANGE",
    -8: "NBG_ERR_NOMEM",
    -9: "NBG_ERR_INDEX",
}

NBG_BC_INFINITE, NBG_BC_CUBIC, NBG_BC_PERIODIC = 0, 1, 2
NBG_SYSTEM_POTENTIAL, NBG_SYSTEM_WATER = 0, 1
NBG_POT_LJ, NBG_POT_EL, NBG_POT_GRAV, NBG_POT_MAG = 1, 2, 4, 8
(NBG_THERMO_NULL, NBG_THERMO_ANDERSEN, NBG_THERMO_BERENDSEN,
 NBG_THERMO_NOSEHOOVER, NBG_THERMO_LANGEVIN) = 0, 1, 2, 3, 4
NBG_FLAG_ALL_PAIRS = 1
NBG_FLAG_GRAV_PLAIN = 2
NBG_FLAG_LANGEVIN_BAOAB = 4

_dp = ctypes.POINTER(ctypes.c_double)
_fp = ctypes.POINTER(ctypes.c_float)


class NbgSystemDesc(ctypes.Structure):
    _fields_ = [
        ("abi_version", ctypes.c_int32),
        ("kind", ctypes.c_int32),
        ("n", ctypes.c_int64),
        ("mass", _dp),
        ("charge", _dp),
        ("dipole", _dp),
        ("potentials", ctypes.c_uint32),
        ("lj_epsilon", ctypes.c_double),
        ("lj_sigma", ctypes.c_double),
        ("lj_cutoff", ctypes.c_double),
        ("el_k", ctypes.c_double),
        ("el_cutoff", ctypes.c_double),
        ("el_eps_rf", ctypes.c_double),
        ("grav_G", ctypes.c_double),
        ("mag_mu_4pi", ctypes.c_double),
        ("water_rOH", ctypes.c_double),
        ("water_aHOH", ctypes.c_double),
        ("water_kb", ctypes.c_double),
        ("water_ka", ctypes.c_double),
        ("bc", ctypes.c_int32),
        ("box", ctypes.c_double * 6),
        ("thermostat", ctypes.c_int32),
        ("thermo_T", ctypes.c_double),
        ("thermo_param", ctypes.c_double),
        ("kb", ctypes.c_double),
        ("seed", ctypes.c_uint64),
        ("skin", ctypes.c_double),
        ("rebuild_every", ctypes.c_int32),
        ("flags", ctypes.c_int32),
    ]


class NbgEnergies(ctypes.Structure):
    _fields_ = [(k, ctypes.c_double) for k in (
        "kinetic", "lennard_jones", "electrostatic", "bonds", "angles", "gravity",
        "potential", "total", "temperature")]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class NbgRunStats(ctypes.Structure):
    _fields_ = [
        ("steps", ctypes.c_int64),
        ("list_builds", ctypes.c_int64),
        ("kernel_launches", ctypes.c_int64),
        ("device_ms", ctypes.c_double),
    ]


class NbgRespaStats(ctypes.Structure):
    _fields_ = [
        ("outer_mts", ctypes.c_int64),
        ("outer_fallback", ctypes.c_int64),
        ("judged", ctypes.c_int64),
        ("judge_mean", ctypes.c_double),
        ("judge_max", ctypes.c_double),
        ("judge_last", ctypes.c_double),
    ]


NBG_ML_NPARAM = 25091
NBG_ML_NTRAIN = 24961
NBG_RESPA_EXACT_SPLIT = 1
NBG_RESPA_NO_FAST_FORCE = 2


class EngineError(RuntimeError):
    """A libnbg call returned a negative nbg_status."""

    def __init__(self, status, message):
        self.status = status
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")


# Every symbol include/nbg.h declares, with (restype, argtypes).
_vp = ctypes.c_void_p
SIGNATURES = {
    "nbg_version": (ctypes.c_char_p, []),
    "nbg_abi_version": (ctypes.c_int, []),
    "nbg_create": (ctypes.c_int, [ctypes.POINTER(NbgSystemDesc), ctypes.c_int, ctypes.POINTER(_vp)]),
    "nbg_create_batch": (ctypes.c_int, [ctypes.POINTER(NbgSystemDesc), ctypes.c_int32, ctypes.c_int,
                                        ctypes.POINTER(_vp)]),
    "nbg_destroy": (None, [_vp]),
    "nbg_last_error": (ctypes.c_char_p, [_vp]),
    "nbg_set_stream": (ctypes.c_int, [_vp, _vp]),
    "nbg_kernel_launches": (ctypes.c_int64, [_vp]),
    "nbg_accel": (ctypes.c_int, [_vp, _dp, _dp, _dp, ctypes.c_double]),
    "nbg_set_state": (ctypes.c_int, [_vp, _dp, _dp]),
    "nbg_get_state": (ctypes.c_int, [_vp, _dp, _dp]),
    "nbg_get_step": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_int64)]),
    "nbg_set_step": (ctypes.c_int, [_vp, ctypes.c_int64]),
    "nbg_compute_forces": (ctypes.c_int, [_vp]),
    "nbg_get_accel": (ctypes.c_int, [_vp, _dp]),
    "nbg_advance": (ctypes.c_int, [_vp, ctypes.c_double, ctypes.c_int64]),
    "nbg_sync": (ctypes.c_int, [_vp]),
    "nbg_run": (ctypes.c_int, [_vp, _dp, _dp, ctypes.c_double, ctypes.c_int64, ctypes.c_int64,
                               _dp, _dp, ctypes.POINTER(NbgRunStats)]),
    "nbg_energy": (ctypes.c_int, [_vp, _dp, _dp, ctypes.POINTER(NbgEnergies)]),
    "nbg_pair_list": (ctypes.c_int, [_vp, _dp, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32),
                                     ctypes.c_int64, ctypes.POINTER(ctypes.c_int64)]),
    "nbg_set_profiling": (ctypes.c_int, [_vp, ctypes.c_int]),
    "nbg_force_kernel_time": (ctypes.c_int, [_vp, _dp, ctypes.POINTER(ctypes.c_int64)]),
    "nbg_force_form": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32)]),
    "nbg_ensemble_form": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32),
                                         ctypes.POINTER(ctypes.c_int32)]),
    "nbg_ensemble_tune": (ctypes.c_int, [_vp, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32), _dp]),
    "nbg_probe_fp32_peak": (ctypes.c_int, [ctypes.c_int, _dp]),
    "nbg_gravity_accel_noalloc": (ctypes.c_int, [_vp, _vp, ctypes.c_int64, ctypes.c_double, _vp, _vp]),
    "nbg_ml_param_count": (ctypes.c_int, []),
    "nbg_ml_enable": (ctypes.c_int, [_vp]),
    "nbg_ml_set_params": (ctypes.c_int, [_vp, ctypes.c_int32, _fp]),
    "nbg_ml_get_params": (ctypes.c_int, [_vp, ctypes.c_int32, _fp]),
    "nbg_ml_init_params": (ctypes.c_int, [_vp, ctypes.c_uint64, ctypes.c_double]),
    "nbg_ml_descriptors": (ctypes.c_int, [_vp, _dp, ctypes.c_int32, _fp]),
    "nbg_ml_eval": (ctypes.c_int, [_vp, _dp, _fp, _dp]),
    "nbg_ml_labels": (ctypes.c_int, [_vp, _dp, _fp, _fp]),
    "nbg_ml_reserve": (ctypes.c_int, [_vp, ctypes.c_int64]),
    "nbg_ml_collect": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_int64)]),
    "nbg_ml_rows": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_int64)]),
    "nbg_ml_normalize": (ctypes.c_int, [_vp]),
    "nbg_ml_train": (ctypes.c_int, [_vp, ctypes.c_int64, ctypes.c_int32, ctypes.c_double, ctypes.c_uint64, _dp]),
    "nbg_ml_batch_gradient": (ctypes.c_int, [_vp, ctypes.c_int32, _fp, _fp, ctypes.c_int32, _fp, _dp]),
    "nbg_respa_run": (ctypes.c_int, [_vp, ctypes.c_double, ctypes.c_int32, ctypes.c_int64, ctypes.c_double,
                                     ctypes.c_int32, ctypes.POINTER(NbgRespaStats)]),
    "nbg_set_thermostat_target": (ctypes.c_int, [_vp, ctypes.c_int32, ctypes.c_double]),
    "nbg_ml_kernel_times": (ctypes.c_int, [_vp, ctypes.c_int32, _dp]),
    "nbg_autotune": (ctypes.c_int, [_vp, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32), _dp]),
    "nbg_cluster_shape": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32)]),
    "nbg_cluster_launch_floor": (ctypes.c_int, [_vp, _dp, _dp]),
    "nbg_rdf_histogram": (ctypes.c_int, [_vp, ctypes.c_int64, ctypes.c_int64, ctypes.POINTER(ctypes.c_int32),
                                         ctypes.c_int64, ctypes.c_double, ctypes.c_int32, ctypes.c_int, _vp]),
    "nbg_rdf_kernel_times": (ctypes.c_int, [_dp]),
}

_lib = None


def load_library(path: str = LIB_PATH):
    """Load libnbg.so and bind its prototypes. Raises if it is missing."""
    global _lib
    if _lib is not None and path == LIB_PATH:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(
            f"{os.path.basename(path)} not found at {path}: build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'` (the debug build with "
            "`python nbodysimulator.jl_gb300/build.py --debug`; the engine has no CPU fallback)")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.nbg_abi_version() != NBG_ABI_VERSION:
        raise RuntimeError("libnbg.so ABI version mismatch")
    if path == LIB_PATH:
        _lib = lib
    return lib


def as_fptr(arr):
    """Pointer to a contiguous float32 numpy array (or None)."""
    if arr is None:
        return None
    return arr.ctypes.data_as(_fp)


def as_dptr(arr):
    """Pointer to a contiguous float64 numpy array (or None)."""
    if arr is None:
        return None
    return arr.ctypes.data_as(_dp)


def rdf_histogram(frames, idx, L, maxbin=1000, device=0, out=None):
    """nbg_rdf_histogram: the reference rdf's pair counts (hist[bin] += 2 per
    pair) over frames of shape (nframes, ncols, 3) for the columns idx.
    frames and out may be numpy arrays or CUDA tensors (data_ptr())."""
    lib = load_library()
    idx = np.ascontiguousarray(idx, dtype=np.int32)
    if hasattr(frames, "data_ptr"):
        nframes, ncols = int(frames.shape[0]), int(frames.shape[1])
        fptr = frames.data_ptr()
    else:
        frames = np.ascontiguousarray(frames, dtype=np.float64)
        nframes, ncols = frames.shape[0], frames.shape[1]
        fptr = frames.ctypes.data
    if out is None:
        out = np.zeros(maxbin)
    optr = out.data_ptr() if hasattr(out, "data_ptr") else out.ctypes.data
    st = lib.nbg_rdf_histogram(fptr, nframes, ncols, idx.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), len(idx),
                               float(L), int(maxbin), int(device), optr)
    if st != NBG_OK:
        raise EngineError(st, "nbg_rdf_histogram")
    return out


def rdf_kernel_times():
    """(split ms, pair-histogram ms) of the last rdf_histogram call."""
    ms = (ctypes.c_double * 2)()
    load_library().nbg_rdf_kernel_times(ms)
    return ms[0], ms[1]
