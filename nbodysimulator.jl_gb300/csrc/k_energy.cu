// k_energy.cu - FP64 energy reductions with the reference's definitions and
// the pair-set export used by the parity tests.
//
// Energies (nbody_simulation_result.jl): kinetic sum m v^2 / 2 (:209-212);
// Lennard-Jones 4 eps sum_{i<j} (s^12 - s^6) with r^2 clamped to R^2 beyond
// the cutoff (:293-319); electrostatic k sum_i q_i sum_{j>i, not excluded}
// (q_j / r or q_j / R) (:321-351); bonds sum over directed bonds k d^2 / 4
// (:353-372); angles sum k (theta - theta0)^2 / 2 (:374-397); gravity
// -G sum_{i<j} m_i m_j / r (this project's; the reference has none).
// Per-block partials are summed by the host in block order (deterministic).
#include "fx_pair.cuh"

#define EB 128

__global__ void __launch_bounds__(EB) k_energy_pairs(Dev d, const double* X, double* out /*[grid][3]*/)
{
    const RepDev& R = d.reps[0];
    double e_lj = 0.0, e_el = 0.0, e_g = 0.0;
    bool range_err = false;
    const bool water = d.kind == NBG_SYSTEM_WATER;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < d.n; i += (int64_t)gridDim.x * blockDim.x) {
        const double* xi = X + 3 * i;
        bool lj_i = (d.pots & NBG_POT_LJ) && (!water || i % 3 == 0);
        double el_i = 0.0, g_i = 0.0;
        for (int64_t j = i + 1; j < d.n; ++j) {
            const double* xj = X + 3 * j;
            bool lj = lj_i && (!water || j % 3 == 0);
            bool el = (d.pots & NBG_POT_EL) && !el_excluded(d.kind, i, j);
            if (lj || el) {
                Dist64 q;
                if (!distance64(xi, xj, d.bc, R, q)) {
                    range_err = true;
                    continue;
                }
                if (lj) {
                    double r2 = q.r2;
                    if (!(r2 < d.lj_R2)) r2 = d.lj_R2;
                    double s6 = d.lj_sig2_d / r2;
                    s6 = __dmul_rn(__dmul_rn(s6, s6), s6);
                    e_lj = __dadd_rn(e_lj, __dsub_rn(__dmul_rn(s6, s6), s6));
                }
                if (el) {
                    if (q.r2 < d.el_R2) {
                        double r = sqrt(q.r2);
                        // reaction field: 1/r + k_rf r^2 - c_rf (+ c_rf back, so eps_rf = 1 gives 1/r)
                        double t = 1.0 / r;
                        if (d.el_krf != 0.0) t = __dadd_rn(t, __dsub_rn(__dmul_rn(d.el_krf, q.r2), d.el_crf - 1.0 / d.el_R));
                        el_i = __dadd_rn(el_i, __dmul_rn(d.charge[j], t));
                    } else {
                        el_i = __dadd_rn(el_i, d.charge[j] / d.el_R);
                    }
                }
            }
            if (d.pots & NBG_POT_GRAV) {
                double x = __dsub_rn(xi[0], xj[0]), y = __dsub_rn(xi[1], xj[1]), z = __dsub_rn(xi[2], xj[2]);
                double r = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z)));
                g_i = __dadd_rn(g_i, d.mass[j] / r);
            }
        }
        if (d.pots & NBG_POT_EL) e_el = __dadd_rn(e_el, __dmul_rn(el_i, d.charge[i]));
        if (d.pots & NBG_POT_GRAV) e_g = __dadd_rn(e_g, __dmul_rn(g_i, d.mass[i]));
    }
    if (range_err) status_set(d.status, ST_RANGE);
    __shared__ double sh[3][EB];
    sh[0][threadIdx.x] = e_lj;
    sh[1][threadIdx.x] = e_el;
    sh[2][threadIdx.x] = e_g;
    __syncthreads();
    for (int w = EB / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w)
            for (int k = 0; k < 3; ++k) sh[k][threadIdx.x] += sh[k][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int k = 0; k < 3; ++k) out[blockIdx.x * 3 + k] = sh[k][0];
}

// The same LJ and electrostatic sums over the Verlet list (built for X):
// for each pair inside a cutoff, its term minus the term the reference gives
// a pair beyond it (LJ at r = R, Coulomb q_i q_j / R); the host adds those
// constant terms for all pairs analytically. O(N x neighbours) instead of
// O(N^2); each pair is taken once (j > i) with the same FP64 minimum image.
__global__ void __launch_bounds__(EB) k_energy_list(Dev d, const double* X, double* out /*[grid][2]*/)
{
    const RepDev& R = d.reps[0];
    double e_lj = 0.0, e_el = 0.0;
    bool range_err = false;
    const bool water = d.kind == NBG_SYSTEM_WATER;
    double s6R = d.lj_sig2_d / d.lj_R2;
    s6R = __dmul_rn(__dmul_rn(s6R, s6R), s6R);
    const double ljR = __dsub_rn(__dmul_rn(s6R, s6R), s6R);
    const double invR = 1.0 / d.el_R;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < d.n; i += (int64_t)gridDim.x * blockDim.x) {
        const double* xi = X + 3 * i;
        const bool lj_i = (d.pots & NBG_POT_LJ) && (!water || i % 3 == 0);
        const int cnt = d.nbr_count[i];
        double el_i = 0.0;
        for (int k = 0; k < cnt; ++k) {
            const int64_t j = dbg_index(d.nbr[(int64_t)k * d.nbr_kstride + i * d.nbr_istride], d.n, (int)i, d.status);
            if (j <= i) continue;
            const bool lj = lj_i && (!water || j % 3 == 0);
            const bool el = (d.pots & NBG_POT_EL) && !el_excluded(d.kind, i, j);
            if (!(lj || el)) continue;
            Dist64 q;
            if (!distance64(xi, X + 3 * j, d.bc, R, q)) {
                range_err = true;
                continue;
            }
            if (lj && q.r2 < d.lj_R2) {
                double s6 = d.lj_sig2_d / q.r2;
                s6 = __dmul_rn(__dmul_rn(s6, s6), s6);
                e_lj = __dadd_rn(e_lj, __dsub_rn(__dsub_rn(__dmul_rn(s6, s6), s6), ljR));
            }
            if (el && q.r2 < d.el_R2) {
                const double r = sqrt(q.r2);
                double t = 1.0 / r;
                if (d.el_krf != 0.0) t = __dadd_rn(t, __dsub_rn(__dmul_rn(d.el_krf, q.r2), d.el_crf - invR));
                el_i = __dadd_rn(el_i, __dmul_rn(d.charge[j], __dsub_rn(t, invR)));
            }
        }
        if (d.pots & NBG_POT_EL) e_el = __dadd_rn(e_el, __dmul_rn(el_i, d.charge[i]));
    }
    if (range_err) status_set(d.status, ST_RANGE);
    __shared__ double sh[2][EB];
    sh[0][threadIdx.x] = e_lj;
    sh[1][threadIdx.x] = e_el;
    __syncthreads();
    for (int w = EB / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w)
            for (int k = 0; k < 2; ++k) sh[k][threadIdx.x] += sh[k][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int k = 0; k < 2; ++k) out[blockIdx.x * 2 + k] = sh[k][0];
}

// kinetic sum (v.v) m/2 and m v.v (temperature), bonds and angles
__global__ void __launch_bounds__(EB) k_energy_local(Dev d, const double* X, const double* V, double* out /*[grid][4]*/)
{
    double ke = 0.0, mv2 = 0.0, eb = 0.0, ea = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < d.n; i += (int64_t)gridDim.x * blockDim.x) {
        double s = __dadd_rn(__dadd_rn(__dmul_rn(V[3 * i], V[3 * i]), __dmul_rn(V[3 * i + 1], V[3 * i + 1])),
                             __dmul_rn(V[3 * i + 2], V[3 * i + 2]));
        ke = __dadd_rn(ke, __dmul_rn(s, d.mass[i] / 2.0));
        mv2 = __dadd_rn(mv2, __dmul_rn(d.mass[i], s));
        if (d.kind == NBG_SYSTEM_WATER && i % 3 == 0) {
            const double *ro = X + 3 * i, *ra = ro + 3, *rc = ro + 6;
            double b1[3], b2[3];
            for (int k = 0; k < 3; ++k) {
                b1[k] = __dsub_rn(ra[k], ro[k]);
                b2[k] = __dsub_rn(rc[k], ro[k]);
            }
            double n1 = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(b1[0], b1[0]), __dmul_rn(b1[1], b1[1])), __dmul_rn(b1[2], b1[2])));
            double n2 = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(b2[0], b2[0]), __dmul_rn(b2[1], b2[1])), __dmul_rn(b2[2], b2[2])));
            double d1 = __dsub_rn(n1, d.rOH), d2 = __dsub_rn(n2, d.rOH);
            // directed bonds O->H1, O->H2, H1->O, H2->O
            double t1 = __dmul_rn(__dmul_rn(d1, d1), d.kbond), t2 = __dmul_rn(__dmul_rn(d2, d2), d.kbond);
            eb = __dadd_rn(eb, __dadd_rn(__dadd_rn(t1, t2), __dadd_rn(t1, t2)));
            double dot = __dadd_rn(__dadd_rn(__dmul_rn(b1[0], b2[0]), __dmul_rn(b1[1], b2[1])), __dmul_rn(b1[2], b2[2]));
            double th = acos(dot / __dmul_rn(n1, n2));
            double dt = __dsub_rn(th, d.aHOH);
            ea = __dadd_rn(ea, __dmul_rn(__dmul_rn(d.kangle, dt), dt));
        }
    }
    __shared__ double sh[4][EB];
    sh[0][threadIdx.x] = ke;
    sh[1][threadIdx.x] = mv2;
    sh[2][threadIdx.x] = eb;
    sh[3][threadIdx.x] = ea;
    __syncthreads();
    for (int w = EB / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w)
            for (int k = 0; k < 4; ++k) sh[k][threadIdx.x] += sh[k][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int k = 0; k < 4; ++k) out[blockIdx.x * 4 + k] = sh[k][0];
}

// out_host: kinetic, lj, el, bonds, angles, gravity, sum m v^2
int launch_energy(nbg_ctx* c, const StateView& s, double* out_host)
{
    const int gp = grid_for(c->n, EB) < 1024 ? grid_for(c->n, EB) : 1024;
    const int gl = grid_for(c->n, EB) < 256 ? grid_for(c->n, EB) : 256;
    double* buf = nullptr;
    size_t bytes = sizeof(double) * (3 * (size_t)gp + 4 * (size_t)gl);
    cudaError_t e = cudaMallocAsync((void**)&buf, bytes, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "energy scratch");
    const bool list = c->path == PATH_LIST && c->nrep == 1;
    if (list) {
        // a list for exactly these positions
        int st = launch_pack(c, s);
        if (st) return st;
        if ((st = launch_list_build(c, s, true, StepRef{0, nullptr}))) return st;
        k_energy_list<<<gp, EB, 0, c->stream>>>(c->d, s.x, buf);
        NBG_LAUNCH_CHECK(c, "k_energy_list");
    } else {
        k_energy_pairs<<<gp, EB, 0, c->stream>>>(c->d, s.x, buf);
        NBG_LAUNCH_CHECK(c, "k_energy_pairs");
    }
    k_energy_local<<<gl, EB, 0, c->stream>>>(c->d, s.x, s.v, buf + 3 * gp);
    NBG_LAUNCH_CHECK(c, "k_energy_local");
    std::vector<double> h(3 * (size_t)gp + 4 * (size_t)gl);
    e = cudaMemcpyAsync(h.data(), buf, bytes, cudaMemcpyDeviceToHost, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "energy copy");
    cudaFreeAsync(buf, c->stream);
    e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "energy sync");
    double lj = 0, el = 0, g = 0, ke = 0, mv2 = 0, eb = 0, ea = 0;
    if (list) {
        for (int b = 0; b < gp; ++b) {
            lj += h[2 * b];
            el += h[2 * b + 1];
        }
        // every pair's beyond-cutoff term: LJ(R) per LJ pair, q_i q_j / R per charge pair
        double s6R = c->d.lj_sig2_d / c->d.lj_R2;
        s6R = s6R * s6R * s6R;
        if (c->d.pots & NBG_POT_LJ) lj += (double)c->lj_pairs * (s6R * s6R - s6R);
        if (c->d.pots & NBG_POT_EL) el += c->el_pair_qq / c->d.el_R;
    } else {
        for (int b = 0; b < gp; ++b) {
            lj += h[3 * b];
            el += h[3 * b + 1];
            g += h[3 * b + 2];
        }
    }
    for (int b = 0; b < gl; ++b) {
        const double* q = h.data() + 3 * gp + 4 * b;
        ke += q[0];
        mv2 += q[1];
        eb += q[2];
        ea += q[3];
    }
    out_host[0] = ke;
    out_host[1] = (c->d.pots & NBG_POT_LJ) ? 4.0 * c->d.lj_eps * lj : 0.0;
    out_host[2] = (c->d.pots & NBG_POT_EL) ? el * c->d.el_k_d : 0.0;
    out_host[3] = c->d.kind == NBG_SYSTEM_WATER ? eb / 4.0 : 0.0;
    out_host[4] = c->d.kind == NBG_SYSTEM_WATER ? ea / 2.0 : 0.0;
    out_host[5] = (c->d.pots & NBG_POT_GRAV) ? -c->d.G * g : 0.0;
    out_host[6] = mv2;
    return NBG_OK;
}

// Pair-set export: every ordered pair the force kernels count as inside the
// cutoff of `which` (NBG_POT_LJ or NBG_POT_EL), same classification code
// (fx: the fixed-point kernel's, fx_pair.cuh; else pair_cutoff's).
__global__ void k_pairs(Dev d, StateView s, int which, int use_list, int fx, int* out_j, int* out_cnt, int64_t cap)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < d.n; i += (int64_t)gridDim.x * blockDim.x) {
        const RepDev& R = d.reps[d.rep_of[i]];
        float4 hi = d.phi[i], lo = d.plo[i];
        int64_t cnt = 0;
        int64_t m = use_list ? d.nbr_count[i] : (R.atom0 + R.n);
        const bool water = d.kind == NBG_SYSTEM_WATER;
        const bool lj_i = (d.pots & NBG_POT_LJ) && (!water || (i % 3) == 0);
        for (int64_t k = use_list ? 0 : R.atom0; k < m; ++k) {
            int64_t j = use_list ? dbg_index(d.nbr[k * d.nbr_kstride + i * d.nbr_istride], d.n, (int)i, d.status) : k;
            if (j == i) continue;
            bool in;
            if (fx) {
                const bool lp = lj_i && (!water || fx_oxygen((int)j));
                const bool ep = (d.pots & NBG_POT_EL) != 0;
                float dx, dy, dz;
                const float r2 = fx_r2(d.pfx[i], d.pfx[j], dx, dy, dz);
                bool lj_in, el_in, amb;
                fx_classify(r2, lp, ep, R.fx_lj_lo, R.fx_lj_hi, R.fx_el_lo, R.fx_el_hi, lj_in, el_in, amb);
                if (amb) {
                    const FxPair o = fx_pair_fallback(d, s.x, i, j, lp, ep);
                    if (o.range_err) status_set(d.status, ST_RANGE);
                    lj_in = o.lj_in;
                    el_in = o.el_in;
                }
                in = which == NBG_POT_LJ ? lj_in : el_in;
            } else {
                PairOut o = pair_cutoff(d, R, PairK(R), i, j, hi, lo, d.phi[j], d.plo[j], 0.0f, s.x);
                if (o.range_err) status_set(d.status, ST_RANGE);
                in = which == NBG_POT_LJ ? o.lj_in : o.el_in;
            }
            if (in) {
                if (cnt < cap) out_j[i * cap + cnt] = (int)j;
                ++cnt;
            }
        }
        out_cnt[i] = (int)cnt;
    }
}

int launch_pairs(nbg_ctx* c, const StateView& s, int which, int* out_j, int* out_cnt, int64_t cap_per_atom)
{
    k_pairs<<<grid_for(c->n, 128), 128, 0, c->stream>>>(c->d, s, which, c->path == PATH_LIST ? 1 : 0,
                                                        c->fx_ready ? 1 : 0, out_j, out_cnt, cap_per_atom);
    NBG_LAUNCH_CHECK(c, "k_pairs");
    return NBG_OK;
}
