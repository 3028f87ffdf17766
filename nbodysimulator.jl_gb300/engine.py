"""Thin object wrapper over one libnbg context (include/nbg.h)."""
import ctypes

import numpy as np

from . import _abi


def _check(lib, ctx, status):
    if status != _abi.NBG_OK:
        msg = lib.nbg_last_error(ctx) if ctx else b""
        raise _abi.EngineError(status, (msg or b"").decode())


def _f64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if shape is not None and a.size != int(np.prod(shape)):
        raise ValueError(f"expected {shape}, got {a.shape}")
    return a


class Engine:
    """A device-resident system (or batch of replicas) on one GPU.

    State arrays are (cols, 3) float64 in memory, i.e. the reference's 3 x n
    column-major layout; cols = n, or n + 1 with the Nose-Hoover column."""

    def __init__(self, descs, device=0):
        self.lib = _abi.load_library()
        ptr = ctypes.c_void_p()
        if isinstance(descs, _abi.NbgSystemDesc):
            descs = [descs]
        arr = (_abi.NbgSystemDesc * len(descs))(*descs)
        if len(descs) == 1:
            st = self.lib.nbg_create(arr, int(device), ctypes.byref(ptr))
        else:
            st = self.lib.nbg_create_batch(arr, len(descs), int(device), ctypes.byref(ptr))
        if st != _abi.NBG_OK:
            raise _abi.EngineError(st, "nbg_create failed")
        self.ctx = ptr
        self.cols = sum(int(d.n) + (1 if d.thermostat == _abi.NBG_THERMO_NOSEHOOVER else 0) for d in descs)

    def _chk(self, st):
        _check(self.lib, self.ctx, st)

    def close(self):
        if getattr(self, "ctx", None):
            self.lib.nbg_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def accel(self, v, u, t=0.0, out=None):
        """soode_system!(dv, v, u, p, t); returns dv (written into `out` when
        given: a C-contiguous float64 array of u's shape, e.g. pinned). With
        Nose-Hoover the thermostat rate is written into v[-1, 0] as in the
        reference."""
        u = _f64(u)
        if out is None:
            dv = np.zeros_like(u)
        else:
            if not (isinstance(out, np.ndarray) and out.dtype == np.float64 and out.flags.c_contiguous
                    and out.shape == u.shape):
                raise TypeError("out must be a C-contiguous float64 array of u's shape")
            dv = out
        if not (isinstance(v, np.ndarray) and v.dtype == np.float64 and v.flags.c_contiguous):
            raise TypeError("v must be a C-contiguous float64 array (it may be written)")
        self._chk(self.lib.nbg_accel(self.ctx, _abi.as_dptr(dv), _abi.as_dptr(v), _abi.as_dptr(u), float(t)))
        return dv

    def set_state(self, u, v):
        u, v = _f64(u), _f64(v)
        self._chk(self.lib.nbg_set_state(self.ctx, _abi.as_dptr(u), _abi.as_dptr(v)))

    def get_state(self):
        u = np.zeros((self.cols, 3))
        v = np.zeros((self.cols, 3))
        self._chk(self.lib.nbg_get_state(self.ctx, _abi.as_dptr(u), _abi.as_dptr(v)))
        return u, v

    def compute_forces(self):
        self._chk(self.lib.nbg_compute_forces(self.ctx))

    def get_accel(self):
        a = np.zeros((self.cols, 3))
        self._chk(self.lib.nbg_get_accel(self.ctx, _abi.as_dptr(a)))
        return a

    def advance(self, dt, nsteps):
        """Queue nsteps on the resident state (asynchronous: the last chunk's
        status is read by the next call, or by sync())."""
        self._chk(self.lib.nbg_advance(self.ctx, float(dt), int(nsteps)))

    def sync(self):
        """Wait for the queued steps; raises the error of the last advance."""
        self._chk(self.lib.nbg_sync(self.ctx))

    @property
    def step(self):
        """The step counter that keys the Andersen / Langevin noise; it keeps
        running across runs (every run draws fresh noise)."""
        out = ctypes.c_int64()
        self._chk(self.lib.nbg_get_step(self.ctx, ctypes.byref(out)))
        return out.value

    def set_step(self, step):
        self._chk(self.lib.nbg_set_step(self.ctx, int(step)))

    def run(self, u, v, dt, nsteps, save_every=0, save_trajectory=True, step=None):
        """Upload (u, v), run, download. Returns (u, v, traj_u, traj_v, stats);
        traj arrays have shape (frames, cols, 3). step: set the noise step
        counter first (None continues it)."""
        if step is not None:
            self.set_step(step)
        u = _f64(u).copy()
        v = _f64(v).copy()
        nframes = (nsteps // save_every + 1 if save_every > 0 else 1) + 1
        tu = np.zeros((nframes, self.cols, 3)) if save_trajectory else None
        tv = np.zeros((nframes, self.cols, 3)) if save_trajectory else None
        stats = _abi.NbgRunStats()
        self._chk(self.lib.nbg_run(self.ctx, _abi.as_dptr(u), _abi.as_dptr(v), float(dt), int(nsteps),
                                   int(save_every), _abi.as_dptr(tu), _abi.as_dptr(tv), ctypes.byref(stats)))
        if save_trajectory:
            used = nsteps // save_every + 1 if save_every > 0 else 1
            if nsteps > 0 and (save_every <= 0 or nsteps % save_every != 0):
                used += 1
            tu, tv = tu[:used], tv[:used]
        return u, v, tu, tv, stats

    def energy(self, u, v):
        out = _abi.NbgEnergies()
        u, v = _f64(u), _f64(v)
        self._chk(self.lib.nbg_energy(self.ctx, _abi.as_dptr(u), _abi.as_dptr(v), ctypes.byref(out)))
        return out.as_dict()

    def pair_list(self, u, which):
        u = _f64(u)
        cnt = ctypes.c_int64()
        self._chk(self.lib.nbg_pair_list(self.ctx, _abi.as_dptr(u), int(which), None, 0, ctypes.byref(cnt)))
        pairs = np.zeros((max(cnt.value, 1), 2), dtype=np.int32)
        self._chk(self.lib.nbg_pair_list(self.ctx, _abi.as_dptr(u), int(which),
                                         pairs.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                         cnt.value, ctypes.byref(cnt)))
        return pairs[: cnt.value]

    def set_stream(self, stream_ptr):
        self._chk(self.lib.nbg_set_stream(self.ctx, ctypes.c_void_p(stream_ptr)))

    def set_profiling(self, on=True):
        self._chk(self.lib.nbg_set_profiling(self.ctx, 1 if on else 0))

    def cluster_launch_floor(self):
        """(µs one launch at a time, µs per launch back to back) of an empty
        kernel with the cluster loop's launch shape, or None off that path."""
        single, b2b = ctypes.c_double(), ctypes.c_double()
        st = self.lib.nbg_cluster_launch_floor(self.ctx, ctypes.byref(single), ctypes.byref(b2b))
        if st == -6:  # NBG_ERR_UNSUPPORTED
            return None
        self._chk(st)
        return single.value, b2b.value

    def cluster_shape(self):
        """(CTAs, lanes per atom) of the persistent cluster step loop, or None
        when the context runs the graph step loop."""
        ctas, lanes = ctypes.c_int32(), ctypes.c_int32()
        used = self.lib.nbg_cluster_shape(self.ctx, ctypes.byref(ctas), ctypes.byref(lanes))
        if used < 0:
            self._chk(used)
        return (ctas.value, lanes.value) if used == 1 else None

    def force_form(self):
        """(lanes per atom, fixed-point list-staged kernel?) of the Verlet-list
        force kernel, or None off the list path."""
        lanes, fx = ctypes.c_int32(), ctypes.c_int32()
        st = self.lib.nbg_force_form(self.ctx, ctypes.byref(lanes), ctypes.byref(fx))
        if st == -6:  # NBG_ERR_UNSUPPORTED: not on the list path
            return None
        self._chk(st)
        return lanes.value, bool(fx.value)

    def ensemble_form(self):
        """(lanes per atom, threads per replica, cells) of the persistent
        ensemble loop, or None when the context does not run it."""
        a, b, c = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        used = self.lib.nbg_ensemble_form(self.ctx, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c))
        if used < 0:
            self._chk(used)
        return (a.value, b.value, c.value) if used == 1 else None

    def ensemble_tune(self, steps=5):
        """Time every form of the ensemble loop and the batch's per-step
        graphs, and keep the fastest; returns ((lanes, threads, cells), or
        None when the graphs win, and the ms per step of the 13 forms)."""
        form = (ctypes.c_int32 * 3)()
        ms = np.zeros(13)
        self._chk(self.lib.nbg_ensemble_tune(self.ctx, int(steps), form, _abi.as_dptr(ms)))
        return ((form[0], form[1], form[2]) if form[0] else None), ms

    def force_kernel_time(self):
        """(summed ms, launches) of the dominant force kernel since the last call."""
        ms = ctypes.c_double()
        cnt = ctypes.c_int64()
        self._chk(self.lib.nbg_force_kernel_time(self.ctx, ctypes.byref(ms), ctypes.byref(cnt)))
        return ms.value, cnt.value

    @property
    def kernel_launches(self):
        return int(self.lib.nbg_kernel_launches(self.ctx))

    # ------------------------------------------------------------------
    # learned short-range model and r-RESPA (SPC/Fw water on the list path)
    # ------------------------------------------------------------------
    def ml_enable(self):
        self._chk(self.lib.nbg_ml_enable(self.ctx))

    def ml_set_params(self, species, theta):
        theta = np.ascontiguousarray(theta, dtype=np.float32)
        if theta.size != _abi.NBG_ML_NPARAM:
            raise ValueError(f"expected {_abi.NBG_ML_NPARAM} parameters, got {theta.size}")
        self._chk(self.lib.nbg_ml_set_params(self.ctx, int(species), _abi.as_fptr(theta)))

    def ml_get_params(self, species):
        theta = np.zeros(_abi.NBG_ML_NPARAM, dtype=np.float32)
        self._chk(self.lib.nbg_ml_get_params(self.ctx, int(species), _abi.as_fptr(theta)))
        return theta

    def ml_init_params(self, seed=0, w1_scale=0.1):
        self._chk(self.lib.nbg_ml_init_params(self.ctx, int(seed), float(w1_scale)))

    def ml_descriptors(self, u, standardised=False):
        u = _f64(u)
        out = np.zeros((u.shape[0], 64), dtype=np.float32)
        self._chk(self.lib.nbg_ml_descriptors(self.ctx, _abi.as_dptr(u), 1 if standardised else 0,
                                              _abi.as_fptr(out)))
        return out

    def ml_eval(self, u):
        """Learned per-atom energies (n,) float32 and forces (n, 3) float64."""
        u = _f64(u)
        e = np.zeros(u.shape[0], dtype=np.float32)
        f = np.zeros((u.shape[0], 3))
        self._chk(self.lib.nbg_ml_eval(self.ctx, _abi.as_dptr(u), _abi.as_fptr(e), _abi.as_dptr(f)))
        return e, f

    def ml_labels(self, u):
        """Exact short-range per-atom energies (n,) and forces (n, 3), float32."""
        u = _f64(u)
        e = np.zeros(u.shape[0], dtype=np.float32)
        f = np.zeros((u.shape[0], 3), dtype=np.float32)
        self._chk(self.lib.nbg_ml_labels(self.ctx, _abi.as_dptr(u), _abi.as_fptr(e), _abi.as_fptr(f)))
        return e, f

    def ml_reserve(self, frames):
        self._chk(self.lib.nbg_ml_reserve(self.ctx, int(frames)))

    def ml_collect(self):
        rows = (ctypes.c_int64 * 2)()
        self._chk(self.lib.nbg_ml_collect(self.ctx, rows))
        return int(rows[0]), int(rows[1])

    def ml_rows(self):
        rows = (ctypes.c_int64 * 2)()
        self._chk(self.lib.nbg_ml_rows(self.ctx, rows))
        return int(rows[0]), int(rows[1])

    def ml_normalize(self):
        self._chk(self.lib.nbg_ml_normalize(self.ctx))

    def ml_train(self, steps, batch=2048, lr=1e-3, seed=0):
        """Adam steps per species; returns the mean loss of the last batches (O, H)."""
        loss = np.zeros(2)
        self._chk(self.lib.nbg_ml_train(self.ctx, int(steps), int(batch), float(lr), int(seed),
                                        _abi.as_dptr(loss)))
        return float(loss[0]), float(loss[1])

    def ml_batch_gradient(self, species, x, y):
        """(loss, gradient of the NBG_ML_NTRAIN trainable parameters) on
        standardised inputs x (B, 64) and targets y (B,)."""
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.float32)
        g = np.zeros(_abi.NBG_ML_NTRAIN, dtype=np.float32)
        loss = ctypes.c_double()
        self._chk(self.lib.nbg_ml_batch_gradient(self.ctx, int(species), _abi.as_fptr(x), _abi.as_fptr(y),
                                                 int(len(y)), _abi.as_fptr(g), ctypes.byref(loss)))
        return loss.value, g

    def respa_run(self, dt, inner, outer, threshold=0.02, exact_split=False, no_fast_force=False):
        """Advance the resident state by `outer` r-RESPA steps; returns the
        stats struct. exact_split: exact short-range force as the fast force;
        no_fast_force: bonded terms only (the integrator's own cost, a ceiling)."""
        stats = _abi.NbgRespaStats()
        flags = _abi.NBG_RESPA_EXACT_SPLIT if exact_split else 0
        if no_fast_force:
            flags = _abi.NBG_RESPA_NO_FAST_FORCE
        self._chk(self.lib.nbg_respa_run(self.ctx, float(dt), int(inner), int(outer), float(threshold), flags,
                                         ctypes.byref(stats)))
        return stats

    def set_thermostat_target(self, T, replica=0):
        self._chk(self.lib.nbg_set_thermostat_target(self.ctx, int(replica), float(T)))

    def ml_kernel_times(self, reps=10):
        """Device ms of (short list, descriptors, MLP, force scatter) on the resident positions."""
        ms = np.zeros(4)
        self._chk(self.lib.nbg_ml_kernel_times(self.ctx, int(reps), _abi.as_dptr(ms)))
        return ms

    def autotune(self, reps=5):
        """Time the list force kernel in every lanes-per-atom form on the resident
        state and keep the fastest; returns (lanes per atom, {form: ms})."""
        lpa = ctypes.c_int32()
        ms = np.zeros(5)
        self._chk(self.lib.nbg_autotune(self.ctx, int(reps), ctypes.byref(lpa), _abi.as_dptr(ms)))
        return lpa.value, dict(zip(("thread", "4", "8", "16", "32"), ms.tolist()))
