// k_ensemble.cu - replica ensembles as one persistent launch per chunk of
// steps: a CTA per replica, the replica's whole step loop inside it.
//
// The replicas of a batch never interact, so no step needs a grid-wide
// barrier: CTA b runs replica order[b] (largest first, so that the big
// replicas start early and the small ones fill the gaps) for all the steps of
// the launch, synchronising only its own threads. Per step:
//   - integration of its atoms (BAOAB for the Langevin thermostat, velocity
//     Verlet without thermostat; the FP64 arithmetic of k_baoab_drift /
//     k_drift_pack) and their fixed-point box coordinates into shared memory
//     (the whole replica: 16 bytes per atom), with the displacement check
//     against the positions of the last list build (fixed point, no FP64);
//   - when a rebuild is due (an atom moved more than skin/2, or
//     rebuild_every steps passed): a counting sort of the atoms into cells in
//     shared memory, each cell's atoms in index order, then every atom's
//     Verlet-list row from the stencil cells (FP32 superset test on the
//     fixed-point differences), written to the global list;
//   - the pair forces of each atom from its list row, gathering neighbours
//     from shared memory (fx_pair2: the fixed-point kernels' classification
//     and arithmetic, so the pair set is the reference's), joined over the
//     atom's lanes, and the velocity update by the group's first lane.
// The Philox noise is keyed (seed, atom, step) as in the step-graph kernels;
// the lists and each replica's steps since its build carry over to the next
// launch unless another path moved the state.
#include <algorithm>
#include <vector>

#include "fx_pair.cuh"

#define ENS_MAX_ATOMS 9216  // largest replica the loop takes (shared memory)
#define ENS_MAX_CELLS 4096

struct EnsArgs {
    const int* order;
    int* since;     // per replica: steps since its build (-1: build first)
    uint4* pref;    // per atom: fixed-point position at its replica's build
    int reuse;      // the lists and counts are this loop's from the previous launch
    int mode;       // cell width: 0 rl / 3^3 stencil, 1 rl/2 / 5^3
    double dt;
    int nsteps;
    int rebuild_every;
    int64_t step0;
    int save;
    int baoab;
};

__device__ __forceinline__ int ens_cell(const uint4& q, int nc)
{
    const int cx = (int)__umulhi(q.x, (unsigned)nc), cy = (int)__umulhi(q.y, (unsigned)nc),
              cz = (int)__umulhi(q.z, (unsigned)nc);
    return (cx * nc + cy) * nc + cz;
}

// Exclusive prefix sum of cnt[0..m) into out[0..m] (out[m] = total), by the
// whole block: a contiguous chunk per thread, then the chunk totals.
template <int THREADS>
__device__ void ens_scan(const int* cnt, int* out, int m, int* warp_tot)
{
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int per = (m + THREADS - 1) / THREADS;
    const int b0 = min(tid * per, m), b1 = min(b0 + per, m);
    int sum = 0;
    for (int k = b0; k < b1; ++k) sum += cnt[k];
    int x = sum;  // inclusive scan in the warp
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[w] = x;
    __syncthreads();
    if (w == 0) {
        int t = lane < THREADS / 32 ? warp_tot[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        if (lane < THREADS / 32) warp_tot[lane] = t;  // inclusive totals of the warps
    }
    __syncthreads();
    int run = x - sum + (w > 0 ? warp_tot[w - 1] : 0);  // exclusive prefix of this thread's chunk
    for (int k = b0; k < b1; ++k) {
        out[k] = run;
        run += cnt[k];
    }
    if (tid == THREADS - 1) out[m] = run;
    __syncthreads();
}

template <int LPA, int POT, int THREADS>
__global__ void __launch_bounds__(THREADS, 1) k_ensemble(Dev d, StateView s, EnsArgs A)
{
    constexpr int G = THREADS / LPA;  // lane groups (atoms in flight)
    const int r = A.order[blockIdx.x];
    const RepDev& R = d.reps[r];
    const int n = (int)R.n;
    const int64_t a0 = R.atom0;
    const int nc = R.ens_nc[A.mode], ns = R.ens_ns[A.mode];
    const int ncell = nc * nc * nc;
    extern __shared__ uint4 ens_sm[];
    uint4* pos = ens_sm;                                   // [n] fixed-point x, y, z and the charge bits
    int* cstart = reinterpret_cast<int*>(pos + n);         // [ncell + 1]
    int* ccur = cstart + (ncell + 1);                      // [ncell]
    int* sorted = ccur + ncell;                            // [n] atoms in cell order
    __shared__ int warp_tot[THREADS / 32];
    const int tid = threadIdx.x, lane = tid % LPA, g = tid / LPA;
    const double dt = A.dt, hdt = 0.5 * dt, dtsq = dt * dt;
    const double c1 = R.bc1;
    const int cap = d.nbr_cap;

    // the frame sink (trajectory saving), read at a save point
    const int64_t sk_every = A.save ? d.sink->every : 0;
    const int64_t sk_t0 = A.save ? d.sink->t0 : 0;
    for (int i = tid; i < n; i += THREADS) pos[i].w = d.pfx[a0 + i].w;
    int since = A.reuse ? A.since[r] : -1;

    bool range_err = false;
    for (int st = 0; st < A.nsteps; ++st) {
        const int64_t step = A.step0 + st;
        // integration to the step's positions, their fixed-point form, and
        // the displacement since the last build
        bool moved = false;
        for (int i = tid; i < n; i += THREADS) {
            const int64_t gi = a0 + i;
            double* x = s.x + 3 * gi;
            double* v = s.v + 3 * gi;
            const double* ao = s.a_old + 3 * gi;
            if (A.baoab) {
                const double sd = __dmul_rn(R.bsd, d.rsqrt_mass[gi]);
                float z[3];
                philox_normals3<float>(R.seed, (uint64_t)i, (uint64_t)step, z);
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const double vh = fma(hdt, ao[k], v[k]);
                    const double xh = fma(hdt, vh, x[k]);
                    const double vo = fma(c1, vh, sd * (double)z[k]);
                    x[k] = fma(hdt, vo, xh);
                    v[k] = vo;
                }
            } else {
#pragma unroll
                for (int k = 0; k < 3; ++k) x[k] = drift1(x[k], v[k], ao[k], dt, dtsq);
            }
            uint4 q = pos[i];
            q.x = fx_coord(x[0], R.fx_scale);
            q.y = fx_coord(x[1], R.fx_scale);
            q.z = fx_coord(x[2], R.fx_scale);
            pos[i] = q;
            if (since >= 0) {
                const uint4 p0 = A.pref[gi];
                float ddx, ddy, ddz;
                const float m2 = fx_r2(q, p0, ddx, ddy, ddz);
                moved |= !(m2 <= R.fx_disp2);
            }
        }
        const bool build = __syncthreads_or(moved ? 1 : 0) || since < 0 ||
                           (A.rebuild_every > 0 && since + 1 >= A.rebuild_every);
        if (build) {
            if (tid == 0) atomicAdd(d.build_count, 1ull);  // the replica's builds, as the graph path counts them
            // counting sort of the atoms into cells, each cell in index order
            for (int c = tid; c < ncell; c += THREADS) ccur[c] = 0;
            __syncthreads();
            for (int i = tid; i < n; i += THREADS) atomicAdd(&ccur[ns > 0 ? ens_cell(pos[i], nc) : 0], 1);
            __syncthreads();
            ens_scan<THREADS>(ccur, cstart, ncell, warp_tot);
            for (int c = tid; c < ncell; c += THREADS) ccur[c] = cstart[c];
            __syncthreads();
            for (int i = tid; i < n; i += THREADS) {
                const int slot = atomicAdd(&ccur[ns > 0 ? ens_cell(pos[i], nc) : 0], 1);
                sorted[slot] = i;
            }
            __syncthreads();
            for (int c = tid; c < ncell; c += THREADS) {  // insertion sort of the cell's atoms
                const int b0 = cstart[c], b1 = cstart[c + 1];
                for (int k = b0 + 1; k < b1; ++k) {
                    const int v0 = sorted[k];
                    int m = k - 1;
                    while (m >= b0 && sorted[m] > v0) {
                        sorted[m + 1] = sorted[m];
                        --m;
                    }
                    sorted[m + 1] = v0;
                }
            }
            __syncthreads();
            // list rows: a warp per cell, lane = one of the cell's atoms (32
            // at a time); the stencil cells' atoms are read once per warp as
            // shared-memory broadcasts, in stencil then index order, and each
            // lane appends those within the list radius to its own row
            {
                const int wid = tid >> 5, wl = tid & 31;
                for (int c = wid; c < ncell; c += THREADS / 32) {
                    const int cx = ns > 0 ? c / (nc * nc) : 0, cy = ns > 0 ? (c / nc) % nc : 0,
                              cz = ns > 0 ? c % nc : 0;
                    const int c0 = cstart[c], c1 = cstart[c + 1];
                    for (int a0c = c0; a0c < c1; a0c += 32) {
                        const bool active = a0c + wl < c1;
                        const int i = active ? sorted[a0c + wl] : 0;
                        const uint4 qi = pos[i];
                        const int64_t gi = a0 + i;
                        int* row = d.nbr + gi * d.nbr_istride;
                        int cnt = 0;
                        for (int ox = -ns; ox <= ns; ++ox) {
                            int nx = cx + ox;
                            nx += nx < 0 ? nc : 0;
                            nx -= nx >= nc ? nc : 0;
                            for (int oy = -ns; oy <= ns; ++oy) {
                                int ny = cy + oy;
                                ny += ny < 0 ? nc : 0;
                                ny -= ny >= nc ? nc : 0;
                                for (int oz = -ns; oz <= ns; ++oz) {
                                    int nz = cz + oz;
                                    nz += nz < 0 ? nc : 0;
                                    nz -= nz >= nc ? nc : 0;
                                    const int cq = (nx * nc + ny) * nc + nz;
                                    const int q1 = cstart[cq + 1];
                                    for (int k = cstart[cq]; k < q1; ++k) {
                                        const int j = sorted[k];
                                        float ddx, ddy, ddz;
                                        if (active && j != i && fx_r2(qi, pos[j], ddx, ddy, ddz) < R.fx_rl2) {
                                            if (cnt < cap) row[(int64_t)cnt * d.nbr_kstride] = (int)(a0 + j);
                                            ++cnt;
                                        }
                                    }
                                }
                            }
                        }
                        if (active) {
                            if (cnt > cap) {
                                status_set(d.status, ST_NBR_OVERFLOW);
                                cnt = cap;
                            }
                            d.nbr_count[gi] = cnt;
                            A.pref[gi] = qi;
                        }
                    }
                }
            }
            since = 0;
            __syncthreads();  // rows written before they are read (other groups)
        } else {
            ++since;
        }
        // forces from the list rows (neighbours from shared memory), then
        // the velocity update of the atom by its group's first lane
        const bool lj_atoms = POT != FX_EL;
        const float lj_lo = R.fx_lj_lo, lj_hi = R.fx_lj_hi, el_lo = R.fx_el_lo, el_hi = R.fx_el_hi;
        const float sig2h = R.fx_sig2_hi, sig2l = R.fx_sig2_lo, krf = R.fx_krf;
        for (int i0 = 0; i0 < n; i0 += G) {
            const int i = i0 + g;
            const bool active = i < n;
            const int64_t gi = a0 + (active ? i : 0);
            const uint4 qi = pos[active ? i : 0];
            const int cnt = active ? min(d.nbr_count[gi], cap) : 0;
            const float kqi =
                POT != FX_LJ ? (float)(d.charge[gi] * R.fx_kq) : 0.0f;
            const int* row = d.nbr + gi * d.nbr_istride;
            float2 px = make_float2(0.f, 0.f), py = px, pz = px;
            // the row entries of the next iteration are loaded before this
            // iteration's gathers and arithmetic (one iteration ahead)
            // (debug builds: an entry outside the replica's atoms is reported
            // and replaced by its first atom before it indexes shared memory)
            int jn0 = lane < cnt ? (int)a0 + dbg_index(__ldg(row + (int64_t)lane * d.nbr_kstride) - (int)a0, n, 0, d.status)
                                 : (int)a0;
            int jn1 = lane + LPA < cnt
                          ? (int)a0 + dbg_index(__ldg(row + (int64_t)(lane + LPA) * d.nbr_kstride) - (int)a0, n, 0, d.status)
                          : jn0;
            for (int k0 = lane; k0 < cnt; k0 += 2 * LPA) {
                const bool v1 = k0 + LPA < cnt;
                const int j0 = jn0, j1 = jn1;
                const int kn = k0 + 2 * LPA;
                jn0 = kn < cnt ? (int)a0 + dbg_index(__ldg(row + (int64_t)kn * d.nbr_kstride) - (int)a0, n, 0, d.status)
                               : (int)a0;
                jn1 = kn + LPA < cnt
                          ? (int)a0 + dbg_index(__ldg(row + (int64_t)(kn + LPA) * d.nbr_kstride) - (int)a0, n, 0, d.status)
                          : jn0;
                const uint4 q0 = pos[j0 - a0], q1 = pos[j1 - a0];
                fx_pair2<POT>(d, s.x, gi, lj_atoms, kqi, qi, j0, j1, true, v1, q0, q1, lj_lo, lj_hi, el_lo, el_hi, sig2h,
                              sig2l, krf, px, py, pz, range_err);
            }
            float hx = __fadd_rn(px.x, px.y), hy = __fadd_rn(py.x, py.y), hz = __fadd_rn(pz.x, pz.y);
            float ex = 0.f, ey = 0.f, ez = 0.f;
#pragma unroll
            for (int o = LPA / 2; o > 0; o >>= 1) {
                fx_join(hx, ex, o, LPA);
                fx_join(hy, ey, o, LPA);
                fx_join(hz, ez, o, LPA);
            }
            if (active && lane == 0) {
                const double im = d.inv_mass[gi] * R.fx_fscale;
                const double an[3] = {((double)hx + (double)ex) * im, ((double)hy + (double)ey) * im,
                                      ((double)hz + (double)ez) * im};
                if (!finite64(an[0]) || !finite64(an[1]) || !finite64(an[2])) status_set(d.status, ST_NONFINITE);
                double* v = s.v + 3 * gi;
                double* ao = s.a_old + 3 * gi;
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    v[k] = A.baoab ? __dadd_rn(v[k], __dmul_rn(hdt, an[k])) : kick1(v[k], ao[k], an[k], dt);
                    ao[k] = an[k];
                    s.a_new[3 * gi + k] = an[k];
                }
                const int64_t t = step + 1 - sk_t0;  // the frame sink's index of the new state
                if (sk_every > 0 && t % sk_every == 0) {
                    const FrameSink* sk = d.sink;
                    const int64_t slot = t / sk_every - sk->first;
                    if (slot >= 0 && slot < sk->cap) {
                        const size_t o = (size_t)slot * 3 * d.cols + 3 * (size_t)gi;
#pragma unroll
                        for (int k = 0; k < 3; ++k) {
                            sk->x[o + k] = s.x[3 * gi + k];
                            sk->v[o + k] = v[k];
                        }
                    }
                }
            }
        }
        __syncthreads();  // the next step's integration overwrites the shared positions
    }
    if (range_err) status_set(d.status, ST_RANGE);
    if (tid == 0) A.since[r] = since;
}

// ---------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------
typedef void (*ens_kernel_t)(Dev, StateView, EnsArgs);

template <int POT, int THREADS>
static ens_kernel_t ens_kernel_lpa(int lpa)
{
    return lpa == 8 ? k_ensemble<8, POT, THREADS> : k_ensemble<4, POT, THREADS>;
}

template <int POT>
static ens_kernel_t ens_kernel_threads(int lpa, int threads)
{
    switch (threads) {
    case 512: return ens_kernel_lpa<POT, 512>(lpa);
    case 1024: return ens_kernel_lpa<POT, 1024>(lpa);
    default: return ens_kernel_lpa<POT, 768>(lpa);
    }
}

static ens_kernel_t ens_kernel(const nbg_ctx* c)
{
    return c->d.pots == NBG_POT_LJ ? ens_kernel_threads<FX_LJ>(c->ens_lpa, c->ens_threads)
                                   : ens_kernel_threads<FX_LJEL>(c->ens_lpa, c->ens_threads);
}

static int ens_mode(const nbg_ctx* c)
{
    return c->ens_cells == 2 ? 1 : 0;
}

// Whether a batch runs the persistent loop, with its form (lanes, threads,
// cell width) and shared memory; per-replica cell grids are set here.
bool ensemble_plan(nbg_ctx* c)
{
    c->ens_ok = false;
    if (c->ens_disabled || c->nrep < 2 || c->path != PATH_LIST || c->d.kind != NBG_SYSTEM_POTENTIAL ||
        c->d.bc != NBG_BC_CUBIC || !c->d.pfx || (c->d.pots & ~(uint32_t)(NBG_POT_LJ | NBG_POT_EL)) ||
        !(c->d.therm == NBG_THERMO_NULL || (c->d.therm == NBG_THERMO_LANGEVIN && c->baoab)))
        return false;
    int64_t nmax = 0;
    int cmax = 1;
    for (int r = 0; r < c->nrep; ++r) {
        RepDev& R = c->reps_h[r];
        nmax = std::max<int64_t>(nmax, R.n);
        const double rl = std::sqrt((double)R.fx_rl2) * (R.L / 4294967296.0);
        const int n1 = (int)std::floor(R.L / (rl * (1.0 + 1e-4)));
        const int n2 = (int)std::floor(R.L / (0.5 * rl * (1.0 + 1e-4)));
        R.ens_nc[0] = n1 >= 3 ? n1 : 1;
        R.ens_ns[0] = n1 >= 3 ? 1 : 0;
        R.ens_nc[1] = n2 >= 5 ? n2 : R.ens_nc[0];
        R.ens_ns[1] = n2 >= 5 ? 2 : R.ens_ns[0];
        for (int m = 0; m < 2; ++m) cmax = std::max(cmax, R.ens_nc[m] * R.ens_nc[m] * R.ens_nc[m]);
    }
    if (nmax > ENS_MAX_ATOMS || cmax > ENS_MAX_CELLS) return false;
    if (cudaMemcpy(const_cast<RepDev*>(c->d.reps), c->reps_h.data(), sizeof(RepDev) * c->nrep,
                   cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    c->ens_smem = sizeof(uint4) * (size_t)nmax + sizeof(int) * (2 * (size_t)cmax + 1 + (size_t)nmax);
    ens_kernel_t k = ens_kernel(c);
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)c->ens_smem) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, c->ens_threads, c->ens_smem) != cudaSuccess || occ < 1) {
        cudaGetLastError();
        return false;
    }
    c->ens_ok = true;
    return true;
}

int launch_ensemble(nbg_ctx* c, const StateView& s, double dt, int64_t nsteps, int64_t step0, unsigned* status)
{
    EnsArgs A;
    A.order = c->ens_order;
    A.since = c->ens_since;
    A.pref = c->ens_pref;
    A.reuse = c->ens_lists_valid ? 1 : 0;
    A.mode = ens_mode(c);
    A.dt = dt;
    A.nsteps = (int)nsteps;
    A.rebuild_every = c->desc.rebuild_every;
    A.step0 = step0;
    A.save = c->sink_on ? 1 : 0;
    A.baoab = c->baoab ? 1 : 0;
    Dev d = c->d;
    d.status = status;
    prof_begin(c);
    ens_kernel(c)<<<(unsigned)c->nrep, (unsigned)c->ens_threads, c->ens_smem, c->stream>>>(d, s, A);
    prof_end(c);
    NBG_LAUNCH_CHECK(c, "k_ensemble");
    return NBG_OK;
}
