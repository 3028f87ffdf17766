"""The debug build (libnbg_debug.so, nvcc -DNBG_DEBUG, loaded with
NBG_DEBUG=1): every neighbour and cell index a kernel reads from a device
table is checked against its range before use, and one outside is reported
as NBG_ERR_INDEX instead of being dereferenced.

- The parity tests of every list-reading kernel (the list force forms, the
  ensemble loop and its step graphs, the cluster loop, the list energies and
  the learned model's short lists) pass unchanged on the debug build: no
  check fires on valid lists, and the checks change no result.
- A planted entry (NBG_TEST_PLANT_INDEX: a debug-build hook that writes an
  index past the end of every per-atom buffer into atom 0's list row after
  the next list build) is caught by each list force kernel form and ends the
  call with NBG_ERR_INDEX; a new context on the same device then runs clean.

Each case runs in a child process, so that the debug library is the only one
it loads."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

# the list force kernel forms: (lanes per atom, extra environment, expected
# nbg_force_form: (lanes, fixed point))
FORMS = {
    "thread_per_atom": (1, {}, (1, False)),
    "split_lanes": (8, {"NBG_NO_FX": "1"}, (8, False)),
    "fixed_point_warp": (4, {}, (4, True)),
    "fixed_point_block": (8, {"NBG_FX_BLOCK": "1"}, (8, True)),
}


@pytest.fixture(scope="module")
def debug_lib(gpu):
    import __graft_entry__ as g
    b = g._load_by_path("nbg_lib_build", os.path.join(ROOT, "nbodysimulator.jl_gb300", "build.py"))
    return b.build(debug=True)


def _run(args, env_extra, timeout=900):
    env = dict(os.environ)
    env.update({"NBG_DEBUG": "1", "PYTHONPATH": os.pathsep.join([HERE, ROOT, env.get("PYTHONPATH", "")])})
    env.update(env_extra)
    return subprocess.run([sys.executable, *args], cwd=ROOT, env=env, capture_output=True, text=True,
                          timeout=timeout)


def test_parity_tests_pass_on_the_debug_build(debug_lib):
    r = _run(["-m", "pytest", "-q", "-x", "-m", "gpu", "-p", "no:cacheprovider",
              "tests/test_gpu_force_forms.py", "tests/test_gpu_ensemble_loop.py",
              "tests/test_gpu_accel_cluster.py", "tests/test_gpu_energy_list.py",
              "tests/test_gpu_learned.py::test_descriptors_match_oracle",
              "tests/test_gpu_learned.py::test_labels_match_oracle",
              "tests/test_gpu_learned.py::test_learned_forces_match_oracle_random_params"], {})
    assert r.returncode == 0, r.stdout[-4000:] + r.stderr[-4000:]
    assert " passed" in r.stdout and " failed" not in r.stdout


def _child_planted(form):
    """(child process) One force evaluation of a 1000-atom LJ liquid with an
    index planted in its list: NBG_ERR_INDEX, then a clean context."""
    import numpy as np

    import systems as S

    nbg = S.nbg
    from nbodysimulator_jl_gb300 import _abi

    assert _abi.LIB_PATH.endswith("libnbg_debug.so")
    lanes, env, expect = FORMS[form]
    sim = S.lj_liquid(1000, seed=21, jitter=0.1)
    desc, keep = nbg.system_descriptor(sim)
    u, v = S.state(sim)
    os.environ.update({"NBG_LIST_LPA": str(lanes), "NBG_NO_CLUSTER": "1", "NBG_TEST_PLANT_INDEX": "7", **env})
    eng = nbg.Engine(desc, 0)
    assert eng.force_form() == expect, eng.force_form()
    eng.set_state(u, v)
    eng.compute_forces()
    try:
        eng.get_accel()
    except _abi.EngineError as e:
        assert e.status == -9, e
    else:
        raise AssertionError("the planted index was not reported")
    eng.close()
    del os.environ["NBG_TEST_PLANT_INDEX"]
    eng = nbg.Engine(desc, 0)
    eng.set_state(u, v)
    eng.compute_forces()
    a = eng.get_accel()
    assert np.all(np.isfinite(a))
    eng.close()
    print("planted index reported:", form)


@pytest.mark.parametrize("form", sorted(FORMS))
def test_planted_list_index_is_reported(debug_lib, form):
    r = _run(["-c", f"import test_gpu_debug_build as t; t._child_planted({form!r})"], {})
    assert r.returncode == 0, r.stdout[-4000:] + r.stderr[-4000:]
    assert "planted index reported" in r.stdout
