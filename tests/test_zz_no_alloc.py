"""nbg_gravity_accel_noalloc: all-pairs gravity for callers that cannot let
a library allocate device memory (a host integrator calling the right-hand
side at a high rate, where cudaMalloc/cudaFree would synchronise the device,
or a process whose device memory belongs to another allocator). It keeps its
scratch in a fixed device array of the library (up to 16384 bodies).

Called through the C ABI on device buffers the test owns, twice in a row
with different sizes (the second call must not see the first call's bodies),
and checked against the context entry point nbg_accel within the force
tolerance of the parity tests."""
import ctypes

import numpy as np
import pytest

import systems as S

nbg = S.nbg
pytestmark = pytest.mark.gpu

FORCE_TOL = 1e-5


def _noalloc(lib, torch, u, m, G):
    x = torch.tensor(np.ascontiguousarray(u), dtype=torch.float64, device="cuda")
    mm = torch.tensor(np.ascontiguousarray(m), dtype=torch.float64, device="cuda")
    a = torch.full_like(x, float("nan"))
    st = lib.nbg_gravity_accel_noalloc(ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(mm.data_ptr()), len(m),
                                       float(G), ctypes.c_void_p(a.data_ptr()), None)
    assert st == 0, lib.nbg_last_error(None)
    return a.cpu().numpy()


def test_noalloc_matches_context_entry_point(gpu):
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    lib = nbg.load_library()
    for n, seed, G in ((3000, 11, 1.0), (1000, 12, 0.5)):
        sim = S.plummer(n, seed=seed)
        sim.system.potentials["gravitational"].G = G
        desc, keep = nbg.system_descriptor(sim)
        u, v = S.state(sim)
        m = np.asarray(keep[0])
        a_ref = nbg.Engine(desc, 0).accel(v.copy(), u)
        a = _noalloc(lib, torch, u, m, G)
        assert np.all(np.isfinite(a))
        assert S.rel_rmse(a, a_ref) <= FORCE_TOL, (n, S.rel_rmse(a, a_ref))


def test_noalloc_rejects_oversize(gpu):
    torch = pytest.importorskip("torch")
    lib = nbg.load_library()
    n = 16385
    x = torch.zeros((n, 3), dtype=torch.float64, device="cuda")
    m = torch.ones(n, dtype=torch.float64, device="cuda")
    a = torch.zeros_like(x)
    st = lib.nbg_gravity_accel_noalloc(ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(m.data_ptr()), n, 1.0,
                                       ctypes.c_void_p(a.data_ptr()), None)
    assert st == -3  # NBG_ERR_CAPACITY
    assert b"16384" in lib.nbg_last_error(None)
