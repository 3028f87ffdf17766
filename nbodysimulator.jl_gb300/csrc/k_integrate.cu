// k_integrate.cu - position packing, the fused velocity-Verlet drift/kick
// with the Berendsen / Nose-Hoover terms, the temperature reduction, the
// Andersen collisions and the Euler-Maruyama Langevin step.
//
// Velocity Verlet is the published method in the form
//   u' = u + dt v + dt^2 (a/2);  a' = f(v, u');  v' = v + dt (a/2 + a'/2)
// where f is soode_system! (nbody_to_ode.jl:474-488) including the
// thermostat terms of thermostats.jl:76-128 evaluated at the start-of-step
// velocity v. All FP64 arithmetic here uses explicit _rn intrinsics so that
// no multiply-add is contracted (the reference's Julia arithmetic has none).
#include <algorithm>

#include "nbg_internal.cuh"

__global__ void k_pack(Dev d, const double* X)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < d.n; i += (int64_t)gridDim.x * blockDim.x)
        pack_atom<true>(d, i, X);
}

int launch_pack(nbg_ctx* c, const StateView& s)
{
    k_pack<<<grid_for(c->n, 256), 256, 0, c->stream>>>(c->d, s.x);
    NBG_LAUNCH_CHECK(c, "k_pack");
    return NBG_OK;
}

// u' = u + dt v + dt^2 (a/2) for one atom's three components, then its split
// position, then the Verlet-list displacement check (moved more than skin/2
// since the last build: flag a rebuild). One thread per atom; the thread after
// the last atom moves the Nose-Hoover column (zeta += dt v_zeta, a = 0).
__global__ void k_drift_pack(Dev d, StateView s, double dt, double dtsq, int check_disp, StepRef pos)
{
    const int parity = (int)(step_of(pos) & 1);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < d.cols; i += (int64_t)gridDim.x * blockDim.x) {
        for (int k = 0; k < 3; ++k) {
            const int64_t e = 3 * i + k;
            s.x[e] = drift1(s.x[e], s.v[e], s.a_old[e], dt, dtsq);
        }
        if (i >= d.n) continue;
        pack_atom(d, i, s.x);
        if (check_disp) {
            double dx = s.x[3 * i] - d.xref[3 * i];
            double dy = s.x[3 * i + 1] - d.xref[3 * i + 1];
            double dz = s.x[3 * i + 2] - d.xref[3 * i + 2];
            double d2 = dx * dx + dy * dy + dz * dz;
            if (!(d2 <= d.skin_half2)) d.rebuild_flag[parity * d.nrep + d.rep_of[i]] = 1;
        }
    }
}

// The rebuild flag written is the one of the positions' time index `pos`.
__global__ void k_pack_disp(Dev d, const double* X, int check_disp, StepRef pos)
{
    const int parity = (int)(step_of(pos) & 1);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < d.n; i += (int64_t)gridDim.x * blockDim.x) {
        pack_atom(d, i, X);
        if (check_disp) {
            double dx = X[3 * i] - d.xref[3 * i];
            double dy = X[3 * i + 1] - d.xref[3 * i + 1];
            double dz = X[3 * i + 2] - d.xref[3 * i + 2];
            double d2 = dx * dx + dy * dy + dz * dz;
            if (!(d2 <= d.skin_half2)) d.rebuild_flag[parity * d.nrep + d.rep_of[i]] = 1;
        }
    }
}

int launch_drift(nbg_ctx* c, const StateView& s, double dt, StepRef pos)
{
    k_drift_pack<<<grid_for(c->cols, 128), 128, 0, c->stream>>>(c->d, s, dt, dt * dt,
                                                                 c->path == PATH_LIST ? 1 : 0, pos);
    NBG_LAUNCH_CHECK(c, "k_drift_pack");
    return NBG_OK;
}

// Per-replica sum of m v^2 (md_temperature, thermostats.jl:87-91), grid
// (slices, replicas); the last block of each replica adds the slice
// partials in slice order, so the result is deterministic.
__global__ void k_temperature(Dev d, const double* V)
{
    int r = blockIdx.y;
    const RepDev& R = d.reps[r];
    int64_t per = (R.n + gridDim.x - 1) / gridDim.x;
    int64_t b = R.atom0 + blockIdx.x * per;
    int64_t e = b + per;
    if (e > R.atom0 + R.n) e = R.atom0 + R.n;
    double acc = 0.0;
    for (int64_t i = b + threadIdx.x; i < e; i += blockDim.x) {
        double sq = V[3 * i] * V[3 * i] + V[3 * i + 1] * V[3 * i + 1] + V[3 * i + 2] * V[3 * i + 2];
        acc += d.mass[i] * sq;
    }
    __shared__ double sh[256];
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    __shared__ bool last;
    if (threadIdx.x == 0) {
        d.red_partial[(int64_t)r * gridDim.x + blockIdx.x] = sh[0];
        __threadfence();
        unsigned prev = atomicAdd(&d.red_counter[r], 1u);
        last = (prev == gridDim.x - 1);
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        __threadfence();
        double tot = 0.0;
        for (int k = 0; k < (int)gridDim.x; ++k) tot += ((volatile double*)d.red_partial)[(int64_t)r * gridDim.x + k];
        d.red_T[r] = tot / (d.kb * R.ndf);
        d.red_counter[r] = 0u;
    }
}

int launch_temperature(nbg_ctx* c, const double* v)
{
    dim3 grid(c->d.red_slices, c->nrep);
    k_temperature<<<grid, 256, 0, c->stream>>>(c->d, v);
    NBG_LAUNCH_CHECK(c, "k_temperature");
    return NBG_OK;
}

// Thermostat term of soode_system! for element e of atom i (i < n) at
// temperature T: Berendsen dv += gamma (T0/T - 1) v (or gamma v when
// 1/T == Inf), Nose-Hoover dv -= zeta v.
__device__ __forceinline__ double thermo_term_T(const Dev& d, int64_t i, double v, double zeta, double T)
{
    if (d.therm == NBG_THERMO_BERENDSEN) {
        const RepDev& R = d.reps[d.rep_of[i]];
        double g = 0.5 / R.tparam;
        if (1.0 / T == INFINITY) return __dmul_rn(g, v);
        return __dmul_rn(__dmul_rn(g, __dsub_rn(R.T0 / T, 1.0)), v);
    }
    if (d.therm == NBG_THERMO_NOSEHOOVER) return -__dmul_rn(zeta, v);
    return 0.0;
}

__device__ __forceinline__ double thermo_term(const Dev& d, int64_t i, double v, double zeta)
{
    return thermo_term_T(d, i, v, zeta, d.red_T[d.rep_of[i]]);
}

// v' = v + dt (a/2 + a'/2) with a' = forces + thermostat term at v; stores a'
// as the next step's a. Also sets the Nose-Hoover rate (thermostats.jl:126).
// With do_T (single system, Berendsen / Nose-Hoover) it also reduces
// sum m v'^2 over the new velocities: block partials, then the last block
// to finish adds them in block order and stores T for the next step's
// thermostat term (every block reads the current T before that).
__global__ void __launch_bounds__(256) k_kick(Dev d, StateView s, double dt, int do_T, int thermo, double* part,
                                              unsigned* counter)
{
    const int64_t ncomp = 3 * d.n;
    double zeta = 0.0;
    if (d.therm == NBG_THERMO_NOSEHOOVER) zeta = s.x[3 * d.n];
    const double T_now = d.red_T[0];
    // Berendsen on a single system: the factor g (T0/T - 1) is the same for
    // every component, so its three FP64 divisions run once per thread (the
    // same operations as thermo_term_T, so the same bits)
    // (one thread per block computes it: an FP64 division is a long
    // sequence on this GPU's FP64 pipe)
    const bool hoist = thermo && d.therm == NBG_THERMO_BERENDSEN && d.nrep == 1;
    double bfac = 0.0;
    if (hoist) {
        __shared__ double bfac_s;
        if (threadIdx.x == 0) {
            const RepDev& R0 = d.reps[0];
            const double T = do_T ? T_now : d.red_T[0];
            const double g = 0.5 / R0.tparam;
            bfac_s = (1.0 / T == INFINITY) ? g : __dmul_rn(g, __dsub_rn(R0.T0 / T, 1.0));
        }
        __syncthreads();
        bfac = bfac_s;
    }
    double acc = 0.0;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < ncomp; e += (int64_t)gridDim.x * blockDim.x) {
        double v = s.v[e];
        double an = s.a_new[e];
        if (hoist)
            an = __dadd_rn(an, __dmul_rn(bfac, v));
        else if (thermo && (d.therm == NBG_THERMO_BERENDSEN || d.therm == NBG_THERMO_NOSEHOOVER))
            an = __dadd_rn(an, thermo_term_T(d, e / 3, v, zeta, do_T ? T_now : d.red_T[d.rep_of[e / 3]]));
        if (!finite64(an)) status_set(d.status, ST_NONFINITE);
        double vn = kick1(v, s.a_old[e], an, dt);
        s.v[e] = vn;
        s.a_old[e] = an;
        if (do_T) acc += d.mass[e / 3] * (vn * vn);
    }
    if (thermo && d.therm == NBG_THERMO_NOSEHOOVER && blockIdx.x == 0 && threadIdx.x < 3) {
        int64_t z = 3 * d.n + threadIdx.x;
        // dv[:, end] = 0; v[zeta] = tau^-2 (T/T0 - (ndf+1)/ndf)
        s.a_old[z] = 0.0;
        if (threadIdx.x == 0) {
            const RepDev& R = d.reps[0];
            double it = 1.0 / R.tparam;
            s.v[z] = __dmul_rn(__dmul_rn(it, it), __dsub_rn(T_now / R.T0, (R.ndf + 1.0) / R.ndf));
        }
    }
    if (!do_T) return;
    __shared__ double sh[256];
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    __shared__ bool last;
    if (threadIdx.x == 0) {
        part[blockIdx.x] = sh[0];
        __threadfence();
        last = (atomicAdd(counter, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    // fixed-order tree over the block partials
    double t = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) t += ((volatile double*)part)[b];
    sh[threadIdx.x] = t;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        d.red_T[0] = sh[0] / (d.kb * d.reps[0].ndf);
        *counter = 0u;
    }
}

int launch_kick(nbg_ctx* c, const StateView& s, double dt, bool do_T, bool thermo)
{
    const int grid = std::min(grid_for(3 * c->n, 256), c->kick_blocks);
    k_kick<<<grid, 256, 0, c->stream>>>(c->d, s, dt, do_T ? 1 : 0, thermo ? 1 : 0, c->kick_part, c->kick_counter);
    NBG_LAUNCH_CHECK(c, "k_kick");
    return NBG_OK;
}

// The thermostat part of one RHS evaluation (nbg_accel): a_new += term(v);
// Nose-Hoover also zeroes its column and writes the rate into v.
__global__ void k_rhs_thermostat(Dev d, StateView s)
{
    int64_t ncomp = 3 * d.n;
    double zeta = d.therm == NBG_THERMO_NOSEHOOVER ? s.x[3 * d.n] : 0.0;
    // Berendsen on a single system: one factor for every component (as in k_kick)
    const bool hoist = d.therm == NBG_THERMO_BERENDSEN && d.nrep == 1;
    double bfac = 0.0;
    if (hoist) {
        __shared__ double bfac_s;
        if (threadIdx.x == 0) {
            const RepDev& R0 = d.reps[0];
            const double T = d.red_T[0];
            const double g = 0.5 / R0.tparam;
            bfac_s = (1.0 / T == INFINITY) ? g : __dmul_rn(g, __dsub_rn(R0.T0 / T, 1.0));
        }
        __syncthreads();
        bfac = bfac_s;
    }
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < ncomp; e += (int64_t)gridDim.x * blockDim.x)
        s.a_new[e] = __dadd_rn(s.a_new[e], hoist ? __dmul_rn(bfac, s.v[e]) : thermo_term(d, e / 3, s.v[e], zeta));
}

__global__ void k_rhs_nh_column(Dev d, StateView s)
{
    int64_t z = 3 * d.n;
    s.a_new[z] = 0.0;
    s.a_new[z + 1] = 0.0;
    s.a_new[z + 2] = 0.0;
    const RepDev& R = d.reps[0];
    double it = 1.0 / R.tparam;
    s.v[z] = __dmul_rn(__dmul_rn(it, it), __dsub_rn(d.red_T[0] / R.T0, (R.ndf + 1.0) / R.ndf));
}

int launch_rhs_thermostat(nbg_ctx* c, const StateView& s)
{
    if (c->d.therm != NBG_THERMO_BERENDSEN && c->d.therm != NBG_THERMO_NOSEHOOVER) return NBG_OK;
    int st = launch_temperature(c, s.v);
    if (st) return st;
    k_rhs_thermostat<<<grid_for(3 * c->n, 256), 256, 0, c->stream>>>(c->d, s);
    NBG_LAUNCH_CHECK(c, "k_rhs_thermostat");
    if (c->d.therm == NBG_THERMO_NOSEHOOVER) {
        k_rhs_nh_column<<<1, 1, 0, c->stream>>>(c->d, s);
        NBG_LAUNCH_CHECK(c, "k_rhs_nh_column");
    }
    return NBG_OK;
}

// Andersen affect! after step `step` (nbody_simulation_result.jl:511-540):
// with probability nu*dt an atom's velocity is redrawn as sqrt(kb T / m) z,
// m = the first body's mass for potential systems, the site mass for water.
__global__ void k_andersen(Dev d, StateView s, double dt, StepRef sr)
{
    const int64_t step = step_of(sr);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < d.n; i += (int64_t)gridDim.x * blockDim.x) {
        int r = d.rep_of[i];
        const RepDev& R = d.reps[r];
        int64_t li = i - R.atom0;
        double prob = R.tparam * dt;
        if (philox_u53(R.seed, (uint64_t)li, (uint64_t)step) < prob) {
            double m = d.kind == NBG_SYSTEM_WATER ? d.mass[i] : d.mass[R.atom0];
            double vdev = sqrt(d.kb * R.T0 / m);
            double z[3];
            philox_normals3<double>(R.seed, (uint64_t)li, (uint64_t)step, z);
            s.v[3 * i] = vdev * z[0];
            s.v[3 * i + 1] = vdev * z[1];
            s.v[3 * i + 2] = vdev * z[2];
        }
    }
}

int launch_andersen(nbg_ctx* c, const StateView& s, double dt, StepRef step)
{
    k_andersen<<<grid_for(c->n, 256), 256, 0, c->stream>>>(c->d, s, dt, step);
    NBG_LAUNCH_CHECK(c, "k_andersen");
    return NBG_OK;
}

// Euler-Maruyama step of the Langevin SDE (nbody_to_ode.jl:567-680):
// u' = u + dt v;  v' = v + dt (a(u) - friction) + sigma sqrt(dt) z.
// Potential systems: friction gamma v, sigma = sqrt(2 gamma kb T / m_1).
// Water (the reference's terms): O rows lose gamma v / m_O and gamma v,
// H rows gamma v; sigma = sqrt(2 gamma kb T) / m_site.
__global__ void k_em(Dev d, StateView s, double dt, double sqdt, StepRef sr)
{
    const int64_t step = step_of(sr);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < d.n; i += (int64_t)gridDim.x * blockDim.x) {
        int r = d.rep_of[i];
        const RepDev& R = d.reps[r];
        int64_t li = i - R.atom0;
        double g = R.tparam;
        float z[3];
        philox_normals3<float>(R.seed, (uint64_t)li, (uint64_t)step, z);
        bool water = d.kind == NBG_SYSTEM_WATER;
        bool oxy = water && (li % 3 == 0);
        double sigma = water ? R.sigma_num / d.mass[i] : R.sigma;
        for (int k = 0; k < 3; ++k) {
            int64_t e = 3 * i + k;
            double v = s.v[e];
            double drift = s.a_new[e];
            if (oxy) drift = __dsub_rn(drift, __dmul_rn(g, v) / d.mass[i]);
            drift = __dsub_rn(drift, __dmul_rn(g, v));
            if (!finite64(drift)) status_set(d.status, ST_NONFINITE);
            double vn = __dadd_rn(__dadd_rn(v, __dmul_rn(dt, drift)), __dmul_rn(sigma, __dmul_rn(sqdt, (double)z[k])));
            s.x[e] = __dadd_rn(s.x[e], __dmul_rn(dt, v));
            s.v[e] = vn;
        }
    }
}

int launch_em(nbg_ctx* c, const StateView& s, double dt, StepRef step)
{
    k_em<<<grid_for(c->n, 128), 128, 0, c->stream>>>(c->d, s, dt, sqrt(dt), step);
    NBG_LAUNCH_CHECK(c, "k_em");
    StepRef pos{step.off + 1, step.base};
    k_pack_disp<<<grid_for(c->n, 256), 256, 0, c->stream>>>(c->d, s.x, c->path == PATH_LIST ? 1 : 0, pos);
    NBG_LAUNCH_CHECK(c, "k_pack_disp");
    return NBG_OK;
}

// BAOAB first half (Leimkuhler & Matthews 2013): B half kick with the old
// forces, A half drift, O exact Ornstein-Uhlenbeck step with each atom's own
// mass, A half drift; then the split position and the displacement check.
__global__ void k_baoab_drift(Dev d, StateView s, double dt, StepRef sr)
{
    const int64_t step = step_of(sr);
    const int parity = (int)((step + 1) & 1);
    const double hdt = 0.5 * dt;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < d.n; i += (int64_t)gridDim.x * blockDim.x) {
        const RepDev& R = d.reps[d.rep_of[i]];
        const int64_t li = i - R.atom0;
        const double c1 = R.bc1;                              // exp(-gamma dt), set by the host for this dt
        const double sd = __dmul_rn(R.bsd, d.rsqrt_mass[i]);  // sqrt(1 - c1^2) sqrt(kb T0 / m)
        float z[3];
        philox_normals3<float>(R.seed, (uint64_t)li, (uint64_t)step, z);
        // fused multiply-adds: FP64 issues slowly on this GPU, and BAOAB has
        // no reference arithmetic to follow operation by operation
        for (int k = 0; k < 3; ++k) {
            const int64_t e = 3 * i + k;
            const double vh = fma(hdt, s.a_old[e], s.v[e]);
            const double x = fma(hdt, vh, s.x[e]);
            const double vo = fma(c1, vh, sd * (double)z[k]);
            s.x[e] = fma(hdt, vo, x);
            s.v[e] = vo;
        }
        pack_atom(d, i, s.x);
        if (d.xref) {
            double dx = s.x[3 * i] - d.xref[3 * i];
            double dy = s.x[3 * i + 1] - d.xref[3 * i + 1];
            double dz = s.x[3 * i + 2] - d.xref[3 * i + 2];
            if (!(dx * dx + dy * dy + dz * dz <= d.skin_half2)) d.rebuild_flag[parity * d.nrep + d.rep_of[i]] = 1;
        }
    }
}

// Inside a captured run of BAOAB steps: the last B of one step (the kick of
// k_baoab_kick) and the B A O A of the next (k_baoab_drift, step sr) in one
// pass over the atoms, with the same operations in the same order, so the
// bits equal the two kernels'. The velocity stays in registers between them.
__global__ void k_baoab_kick_drift(Dev d, StateView s, double dt, StepRef sr)
{
    const int64_t step = step_of(sr);
    const int parity = (int)((step + 1) & 1);
    const double hdt = 0.5 * dt;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < d.n; i += (int64_t)gridDim.x * blockDim.x) {
        const RepDev& R = d.reps[d.rep_of[i]];
        const int64_t li = i - R.atom0;
        const double c1 = R.bc1;
        const double sd = __dmul_rn(R.bsd, d.rsqrt_mass[i]);
        float z[3];
        philox_normals3<float>(R.seed, (uint64_t)li, (uint64_t)step, z);
        for (int k = 0; k < 3; ++k) {
            const int64_t e = 3 * i + k;
            const double an = s.a_new[e];
            if (!finite64(an)) status_set(d.status, ST_NONFINITE);
            const double v = __dadd_rn(s.v[e], __dmul_rn(hdt, an));
            s.a_old[e] = an;
            const double vh = fma(hdt, an, v);
            const double x = fma(hdt, vh, s.x[e]);
            const double vo = fma(c1, vh, sd * (double)z[k]);
            s.x[e] = fma(hdt, vo, x);
            s.v[e] = vo;
        }
        pack_atom(d, i, s.x);
        if (d.xref) {
            double dx = s.x[3 * i] - d.xref[3 * i];
            double dy = s.x[3 * i + 1] - d.xref[3 * i + 1];
            double dz = s.x[3 * i + 2] - d.xref[3 * i + 2];
            if (!(dx * dx + dy * dy + dz * dz <= d.skin_half2)) d.rebuild_flag[parity * d.nrep + d.rep_of[i]] = 1;
        }
    }
}

int launch_baoab_kick_drift(nbg_ctx* c, const StateView& s, double dt, StepRef step)
{
    k_baoab_kick_drift<<<grid_for(c->n, 128), 128, 0, c->stream>>>(c->d, s, dt, step);
    NBG_LAUNCH_CHECK(c, "k_baoab_kick_drift");
    return NBG_OK;
}

// BAOAB last B: v += dt/2 a(x'); the new forces become the next step's.
__global__ void k_baoab_kick(Dev d, StateView s, double dt)
{
    const double hdt = 0.5 * dt;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < 3 * d.n; e += (int64_t)gridDim.x * blockDim.x) {
        double an = s.a_new[e];
        if (!finite64(an)) status_set(d.status, ST_NONFINITE);
        s.v[e] = __dadd_rn(s.v[e], __dmul_rn(hdt, an));
        s.a_old[e] = an;
    }
}

int launch_baoab_drift(nbg_ctx* c, const StateView& s, double dt, StepRef step)
{
    k_baoab_drift<<<grid_for(c->n, 128), 128, 0, c->stream>>>(c->d, s, dt, step);
    NBG_LAUNCH_CHECK(c, "k_baoab_drift");
    return NBG_OK;
}

int launch_baoab_kick(nbg_ctx* c, const StateView& s, double dt)
{
    k_baoab_kick<<<grid_for(3 * c->n, 256), 256, 0, c->stream>>>(c->d, s, dt);
    NBG_LAUNCH_CHECK(c, "k_baoab_kick");
    return NBG_OK;
}

// After the step with StepRef sr: when its new time index t is a save point
// of the sink, copy the state (positions and velocities) into its slot.
__global__ void k_save_frame(const FrameSink* sink, const double* x, const double* v, int64_t n3, StepRef sr)
{
    const int64_t every = sink->every;
    if (every <= 0) return;
    const int64_t t = (sr.base ? *sr.base : 0) + sr.off + 1 - sink->t0;
    if (t % every != 0) return;
    const int64_t slot = t / every - sink->first;
    if (slot < 0 || slot >= sink->cap) return;
    double* fx = sink->x + slot * n3;
    double* fv = sink->v + slot * n3;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n3; i += (int64_t)gridDim.x * blockDim.x) {
        fx[i] = x[i];
        fv[i] = v[i];
    }
}

int launch_save_frame(nbg_ctx* c, const StateView& s, StepRef sr)
{
    const int64_t n3 = 3 * c->d.cols;
    k_save_frame<<<grid_for(n3, 256), 256, 0, c->stream>>>(c->d.sink, s.x, s.v, n3, sr);
    NBG_LAUNCH_CHECK(c, "k_save_frame");
    return NBG_OK;
}

__global__ void k_step_advance(int64_t* step, int64_t by) { *step += by; }
__global__ void k_set_step(int64_t* step, int64_t value) { *step = value; }

int launch_step_advance(nbg_ctx* c, int64_t by)
{
    k_step_advance<<<1, 1, 0, c->stream>>>(c->d.step_dev, by);
    NBG_LAUNCH_CHECK(c, "k_step_advance");
    return NBG_OK;
}

// The right-hand side's first node: u (and v) read from the caller-facing
// pinned staging (host memory the GPU reads directly), stored into the
// scratch state, packed, and checked for displacement against the positions
// of the last list build (rebuild flag of the call counter's parity); the
// status word starts clean.
__global__ void k_accel_import(Dev d, StateView s, const double* __restrict__ hu, const double* __restrict__ hv,
                               int v_read, StepRef pos)
{
    if (blockIdx.x == 0 && threadIdx.x == 0) *d.status = 0u;
    const int parity = (int)(step_of(pos) & 1);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < d.cols; i += (int64_t)gridDim.x * blockDim.x) {
        for (int k = 0; k < 3; ++k) {
            s.x[3 * i + k] = hu[3 * i + k];
            if (v_read) s.v[3 * i + k] = hv[3 * i + k];
        }
        if (i >= d.n) continue;
        pack_atom(d, i, s.x);
        const double dx = s.x[3 * i] - d.xref[3 * i];
        const double dy = s.x[3 * i + 1] - d.xref[3 * i + 1];
        const double dz = s.x[3 * i + 2] - d.xref[3 * i + 2];
        if (!(dx * dx + dy * dy + dz * dz <= d.skin_half2)) d.rebuild_flag[parity * d.nrep + d.rep_of[i]] = 1;
    }
}

// The right-hand side's last node: dv (and the Nose-Hoover rate) and the
// status word written straight into the pinned staging; the call counter
// advances.
__global__ void k_accel_export(Dev d, StateView s, double* __restrict__ hdv, double* __restrict__ hv, unsigned* hstat,
                               int64_t* counter, int nh)
{
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < 3 * d.cols; e += (int64_t)gridDim.x * blockDim.x)
        hdv[e] = s.a_new[e];
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (nh) hv[3 * d.n] = s.v[3 * d.n];
        *hstat = *d.status;
        *counter += 1;
    }
}

int launch_accel_import(nbg_ctx* c, const StateView& s, const double* hu, const double* hv, bool v_read, StepRef pos)
{
    k_accel_import<<<grid_for(c->cols, 256), 256, 0, c->stream>>>(c->d, s, hu, hv, v_read ? 1 : 0, pos);
    NBG_LAUNCH_CHECK(c, "k_accel_import");
    return NBG_OK;
}

int launch_accel_export(nbg_ctx* c, const StateView& s, double* hdv, double* hv, unsigned* hstat, int64_t* counter)
{
    k_accel_export<<<grid_for(3 * c->cols, 256), 256, 0, c->stream>>>(c->d, s, hdv, hv, hstat, counter,
                                                                      c->d.therm == NBG_THERMO_NOSEHOOVER ? 1 : 0);
    NBG_LAUNCH_CHECK(c, "k_accel_export");
    return NBG_OK;
}

int launch_counter_advance(nbg_ctx* c, int64_t* counter, int64_t by)
{
    k_step_advance<<<1, 1, 0, c->stream>>>(counter, by);
    NBG_LAUNCH_CHECK(c, "k_step_advance");
    return NBG_OK;
}

int launch_pack_disp(nbg_ctx* c, const double* X, StepRef pos)
{
    k_pack_disp<<<grid_for(c->n, 256), 256, 0, c->stream>>>(c->d, X, c->path == PATH_LIST ? 1 : 0, pos);
    NBG_LAUNCH_CHECK(c, "k_pack_disp");
    return NBG_OK;
}

int launch_set_step(nbg_ctx* c, int64_t value)
{
    k_set_step<<<1, 1, 0, c->stream>>>(c->d.step_dev, value);
    NBG_LAUNCH_CHECK(c, "k_set_step");
    return NBG_OK;
}
