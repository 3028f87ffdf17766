// k_cluster.cu - velocity Verlet for small systems (up to 2048 atoms) as one
// persistent launch over a thread-block cluster.
//
// A step of a small system is a handful of microsecond kernels, so launches,
// not arithmetic, set its pace. Here the cluster's CTAs (up to 16 SMs) run
// many steps in one launch:
//   - CTA r owns atoms [r per, (r+1) per); its threads drift them (FP64, the
//     reference's velocity-Verlet arithmetic) and split the new positions
//     into its shared memory, in the buffer of the step's parity; one thread
//     sends the contiguous range to every other CTA's same buffer as two bulk
//     asynchronous copies (cp.async.bulk, distributed shared memory), which
//     complete as transaction bytes on the receiver's mbarrier of that parity;
//   - one cluster barrier per step (release/acquire) orders the rebuild flags
//     and the FP64 copies, then every CTA waits (bounded) for its mbarrier;
//     with two parity buffers, a copy of step s+2 can only start after the
//     barrier of step s+1, when every CTA is done reading step s;
//   - each CTA keeps the Verlet lists of its own atoms in shared memory,
//     rebuilt from the shared positions (all atoms scanned, the FP32 superset
//     test of the list builders) when any atom moved more than skin/2 since
//     the last build and every rebuild_every steps; a launch that built
//     them stores them at its end (the steps since the build always), and
//     the next one starts from them unless the host invalidated them (a new
//     state), else it builds first;
//   - at its start a launch writes x, v, a_old of its atoms to the backup,
//     from which the host undoes a launch that timed out or overflowed;
//   - LPA lanes per atom evaluate the pairs (pair_cutoff: the exact pair set;
//     the ambiguous ones read FP64 positions, which the drift also writes to
//     a global copy of the step's parity, through L2) and join their
//     partials (compensated FP32) into shared memory; the atom's owner thread,
//     which keeps its x, v, a in registers for the whole launch, kicks the
//     velocity at the start of the next step.
// Every thread of every CTA passes the same cluster barriers (no early exit).
//
// The same kernel with ACCEL evaluates the right-hand side alone (nbg_accel):
// the positions come from src (pinned host memory read over the CPU-GPU
// link, or device memory), one step of the loop without drift or kick runs
// (exchange, displacement check, list build when needed, forces), and the
// accelerations go to dst; the lists it keeps are its own, built for earlier
// calls' positions, and the resident state is not touched.
#include <algorithm>

#include <cooperative_groups.h>

#include "nbg_internal.cuh"

namespace cg = cooperative_groups;

#define CL_THREADS 1024
#define CL_MAX 16

// mbarrier and bulk-copy helpers (shared-memory addresses as 32-bit
// shared-window offsets; remote ones from mapa)
__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned cluster_addr(unsigned a, int rank)
{
    unsigned r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
    return r;
}

__device__ __forceinline__ void mbar_init(unsigned a, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned a, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(a), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned a, unsigned parity)
{
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    return ok != 0;
}

// bytes (a multiple of 16, 16-byte aligned ends) of this CTA's shared memory
// to another CTA's, completing as transaction bytes on that CTA's mbarrier
__device__ __forceinline__ void bulk_copy_to_peer(unsigned dst_cluster, unsigned src, unsigned bytes,
                                                  unsigned mbar_cluster)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.shared::cta.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            dst_cluster),
        "r"(src), "r"(bytes), "r"(mbar_cluster)
        : "memory");
}

#define CL_WAIT_TRIES (1u << 16)

// (h, e) += the partner lane's (h, e), h by TwoSum with its error into e
__device__ __forceinline__ void cl_join(float& h, float& e, int o, int width)
{
    const float h2 = __shfl_xor_sync(0xffffffffu, h, o, width);
    const float e2 = __shfl_xor_sync(0xffffffffu, e, o, width);
    float sum, err;
    two_sum(h, h2, sum, err);
    h = sum;
    e = __fadd_rn(__fadd_rn(e, e2), err);
}

// Shared memory (dynamic): split positions [parity][hi, lo][n] (float4), the
// own atoms' positions at the last list build [per][3] (double, padded to a 16-byte end), their lists
// [per][cap], counts [per] (int) and force partials [per][6] (float: h, e per
// component).
template <int LPA, bool ACCEL>
__global__ void __launch_bounds__(CL_THREADS, 1) k_cluster_vv(Dev d, StateView s, double* xb, double dt, int nsteps,
                                                              int rebuild_every, int per, int cap, int* lst_g,
                                                              int* cnt_g, double* xref_g, int* since_g, int reuse,
                                                              int64_t step0, int save, int drop_step,
                                                              double* __restrict__ bk,
                                                              const double* __restrict__ src, double* __restrict__ dst)
{
    cg::cluster_group cl = cg::this_cluster();
    const int rank = (int)cl.block_rank();
    const int C = (int)cl.num_blocks();
    const int n = (int)d.n;
    extern __shared__ float4 cl_pos[];
    double* xref_s = reinterpret_cast<double*>(cl_pos + 4 * (size_t)n);
    int* lst = reinterpret_cast<int*>(xref_s + 3 * (size_t)per + ((3 * per) & 1));  // 16-byte aligned
    int* cnt = lst + (size_t)per * cap;
    float* fsum = reinterpret_cast<float*>(cnt + per);
    __shared__ unsigned flag[2];  // rebuild requests of the step of each parity
    __shared__ int build_s;
    __shared__ __align__(8) unsigned long long mbar[2];  // other CTAs' positions of each parity arrived
    __shared__ int wait_failed;  // a bounded wait of this CTA ran out (this step)
    __shared__ int abort_s;      // some CTA's wait ran out: every CTA leaves after the next cluster barrier
    const RepDev& R = d.reps[0];
    const PairK K(R);
    const int tid = threadIdx.x;
    const int a0 = rank * per;
    const int na = max(0, min(n - a0, per));
    const int g = tid / LPA, lane = tid % LPA;  // lane group g <-> own atom a0 + g
    const unsigned gshift = (unsigned)((tid & 31) / LPA * LPA);
    const unsigned gmask = (LPA == 32 ? 0xffffffffu : ((1u << LPA) - 1u));
    const double dtsq = dt * dt;
    const float magic = 12582912.0f;  // 1.5 * 2^23: rint by addition

    // own atom k = tid keeps its state in the registers of thread k for the
    // whole launch
    const int ko = tid;
    const bool owner = tid < na;
    const int io = owner ? a0 + ko : 0;
    double x[3], v[3], a[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        x[k] = owner ? (ACCEL ? src[3 * io + k] : s.x[3 * io + k]) : 0.0;
        v[k] = owner && !ACCEL ? s.v[3 * io + k] : 0.0;
        a[k] = owner && !ACCEL ? s.a_old[3 * io + k] : 0.0;
    }
    const double im_o = owner ? d.inv_mass[io] : 0.0;
    if (owner && !ACCEL) {
        // the backup of the launch's start (x, v, a_old segments of 3 cols):
        // a timed-out or overflowed launch is undone from it
        const size_t seg = 3 * (size_t)d.cols;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            bk[3 * io + k] = x[k];
            bk[seg + 3 * io + k] = v[k];
            bk[2 * seg + 3 * io + k] = a[k];
        }
    }

    // the static w parts (charge, atom flags) of every atom in both parities
    for (int j = tid; j < n; j += CL_THREADS) {
        const float wh = d.phi[j].w, wl = d.plo[j].w;
        for (int p = 0; p < 2; ++p) {
            cl_pos[(2 * p) * (size_t)n + j].w = wh;
            cl_pos[(2 * p + 1) * (size_t)n + j].w = wl;
        }
    }
    int since = 0;
    bool built = false;  // a list build ran in this launch (the same in every CTA)
    if (reuse) {
        // the lists, their reference positions and the steps since their
        // build, as the previous launch left them
        // (cap is a multiple of 4: whole 16-byte rows, several loads in flight per thread)
        const int4* src4 = reinterpret_cast<const int4*>(lst_g + (size_t)rank * per * cap);
        int4* dst4 = reinterpret_cast<int4*>(lst);
#pragma unroll 4
        for (int t = tid; t < na * cap / 4; t += CL_THREADS) dst4[t] = src4[t];
        for (int t = tid; t < na; t += CL_THREADS) cnt[t] = cnt_g[(size_t)rank * per + t];
        for (int t = tid; t < 3 * na; t += CL_THREADS) xref_s[t] = xref_g[3 * (size_t)a0 + t];
        since = *since_g;
    }
    if (tid < 2) flag[tid] = 0u;
    if (tid == 0) {
        wait_failed = 0;
        abort_s = 0;
        mbar_init(smem_addr(&mbar[0]), 1);
        mbar_init(smem_addr(&mbar[1]), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // every CTA of the cluster is running (and initialised) before any
    // remote shared-memory access
    cl.sync();

    // the frame sink (trajectory saving): state of time index step0 + st;
    // its other fields are read at a save point
    const int64_t sk_every = save && owner ? d.sink->every : 0;
    const int64_t sk_t0 = save && owner ? d.sink->t0 : 0;

    for (int st = 0; st <= nsteps; ++st) {
        // kick of the previous step with the forces its groups left in fsum
        if constexpr (ACCEL) {
            if (owner && st > 0) {
                // the right-hand side: the acceleration of the source positions
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const double an = ((double)fsum[6 * ko + 2 * k] + (double)fsum[6 * ko + 2 * k + 1]) * im_o;
                    if (!finite64(an)) status_set(d.status, ST_NONFINITE);
                    dst[3 * io + k] = an;
                }
            }
        } else if (owner && st > 0) {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const double an = ((double)fsum[6 * ko + 2 * k] + (double)fsum[6 * ko + 2 * k + 1]) * im_o;
                if (!finite64(an)) status_set(d.status, ST_NONFINITE);
                v[k] = kick1(v[k], a[k], an, dt);
                a[k] = an;
            }
            if (sk_every > 0 && (step0 + st - sk_t0) % sk_every == 0) {
                const FrameSink* sk = d.sink;
                const int64_t slot = (step0 + st - sk_t0) / sk_every - sk->first;
                if (slot >= 0 && slot < sk->cap) {
                    const size_t o = (size_t)slot * 3 * d.cols + 3 * (size_t)io;
                    double* fx = sk->x;
                    double* fv = sk->v;
#pragma unroll
                    for (int k = 0; k < 3; ++k) {
                        fx[o + k] = x[k];
                        fv[o + k] = v[k];
                    }
                }
            }
        }
        if (st == nsteps) break;  // uniform: every thread leaves after the last kick
        const int par = st & 1;
        float4* ph = cl_pos + (2 * par) * (size_t)n;
        float4* pl = ph + n;
        double* X = xb + (size_t)par * 3 * n;  // FP64 positions of this step
        // drift, split and displacement check of the own atoms
        bool moved = false;
        if (owner) {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                if (!ACCEL) x[k] = drift1(x[k], v[k], a[k], dt, dtsq);
                X[3 * io + k] = x[k];
            }
            float h[3], l[3];
            split_position(d, R, x, h, l);
            ph[io] = make_float4(h[0], h[1], h[2], ph[io].w);
            pl[io] = make_float4(l[0], l[1], l[2], pl[io].w);
            // (a launch that does not reuse lists builds at step 0, which
            // sets xref_s)
            const double* xr = xref_s + 3 * ko;
            const double dx = x[0] - xr[0], dy = x[1] - xr[1], dz = x[2] - xr[2];
            moved = (st > 0 || reuse) && !(dx * dx + dy * dy + dz * dz <= d.skin_half2);
        }
        // the owners' generic writes become visible to the bulk-copy engine
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        const int any_moved = __syncthreads_or(moved ? 1 : 0);
        // the own atoms' split positions (contiguous hi and lo ranges) go to
        // every other CTA as two bulk copies each, completing on its mbarrier
        // of this parity; this CTA expects the other (n - na) atoms' 32 bytes
        if (tid == 0) {
            const unsigned mb = smem_addr(&mbar[par]);
            mbar_arrive_expect_tx(mb, (unsigned)(n - na) * 32u);
            // (drop_step: a host-set test of the timeout path; no CTA sends
            // that step's positions, so its waits run out with nothing in flight)
            if (na > 0 && st != drop_step) {
                const unsigned sh = smem_addr(ph + a0), sl = smem_addr(pl + a0), bytes = (unsigned)na * 16u;
                for (int r = 0; r < C; ++r) {
                    if (r == rank) continue;
                    const unsigned rmb = cluster_addr(mb, r);
                    bulk_copy_to_peer(cluster_addr(sh, r), sh, bytes, rmb);
                    bulk_copy_to_peer(cluster_addr(sl, r), sl, bytes, rmb);
                }
            }
        }
        if (any_moved && tid < C) *cl.map_shared_rank(&flag[par], tid) = 1u;
        // arrive (release) / wait (acquire) at cluster scope: the rebuild
        // flags, the FP64 copies X and an abort raised in the previous step
        // are visible past it
        cl.sync();
        const unsigned mb_cur = smem_addr(&mbar[par]), phase_cur = (unsigned)((st >> 1) & 1);
        if (abort_s) {
            // every CTA saw the same flag after the same barrier: leave the
            // step loop together, once this step's incoming copies (sent
            // before the barrier) have landed (bounded)
            unsigned tries = 0;
            while (!mbar_try_wait(mb_cur, phase_cur) && ++tries < CL_WAIT_TRIES) {
            }
            break;
        }
        // the other CTAs' positions of this step: the k-th use of mbar[par]
        // completes phase k (bounded wait; a timeout is reported as
        // ST_TIMEOUT and ends the launch at the next cluster barrier)
        {
            unsigned tries = 0;
            while (!mbar_try_wait(mb_cur, phase_cur)) {
                if (++tries >= CL_WAIT_TRIES) {
                    wait_failed = 1;
                    break;
                }
            }
        }
        __syncthreads();
        if (tid == 0 && wait_failed) {
            status_set(d.status, ST_TIMEOUT);
            for (int r = 0; r < C; ++r) *cl.map_shared_rank(&abort_s, r) = 1;
        }
        if (tid == 0) {
            build_s = ((st == 0 && !reuse) || flag[par] != 0u || (rebuild_every > 0 && since >= rebuild_every)) ? 1 : 0;
            // the next writes to flag[par] come at step st + 2, after the
            // barrier of step st + 1, which this CTA passes only later
            flag[par] = 0u;
        }
        __syncthreads();
        if (build_s) {
            // lists of the own atoms: group g scans every atom j (lane-strided),
            // entries in j order (ballot-compacted)
            const bool active = g < na;
            const int i = active ? a0 + g : 0;
            const float4 hi = ph[i];
            int c0 = 0;
            for (int jb = 0; jb < n; jb += LPA) {
                const int j = jb + lane;
                bool take = false;
                if (active && j < n && j != i) {
                    const float4 hj = ph[j];
                    float dx = hj.x - hi.x, dy = hj.y - hi.y, dz = hj.z - hi.z;
                    dx = __fmaf_rn(-__fsub_rn(__fmaf_rn(dx, R.invLf, magic), magic), R.Lh, dx);
                    dy = __fmaf_rn(-__fsub_rn(__fmaf_rn(dy, R.invLf, magic), magic), R.Lh, dy);
                    dz = __fmaf_rn(-__fsub_rn(__fmaf_rn(dz, R.invLf, magic), magic), R.Lh, dz);
                    take = dx * dx + dy * dy + dz * dz < R.rl2;
                }
                const unsigned m = (__ballot_sync(0xffffffffu, take) >> gshift) & gmask;
                if (take) {
                    const int q = c0 + __popc(m & ((1u << lane) - 1u));
                    if (q < cap) lst[g * cap + q] = j;
                }
                c0 += __popc(m);
            }
            if (active && lane == 0) {
                if (c0 > cap) {
                    status_set(d.status, ST_NBR_OVERFLOW);
                    c0 = cap;
                }
                cnt[g] = c0;
            }
            if (owner) {
#pragma unroll
                for (int k = 0; k < 3; ++k) xref_s[3 * ko + k] = x[k];
            }
            since = 0;
            built = true;
            __syncthreads();
        }
        ++since;
        // forces of the own atoms: FP32 partials joined over the group, left
        // in fsum for the owner's kick
        {
            const bool active = g < na;
            const int i = active ? a0 + g : 0;
            const float4 hi_i = ph[i], lo_i = pl[i];
            const float kqi = (d.pots & NBG_POT_EL) ? (float)(d.el_k_d * d.charge[i]) : 0.0f;
            const int c = active ? cnt[g] : 0;
            float px = 0.f, py = 0.f, pz = 0.f;
            bool range_err = false;
            for (int k = lane; k < c; k += LPA) {
                const int j = dbg_index(lst[g * cap + k], d.n, i, d.status);
                const PairOut o = pair_cutoff<true>(d, R, K, i, j, hi_i, lo_i, ph[j], pl[j], kqi, X);
                range_err |= o.range_err;
                px += o.fx;
                py += o.fy;
                pz += o.fz;
            }
            float ex = 0.f, ey = 0.f, ez = 0.f;
#pragma unroll
            for (int o = LPA / 2; o > 0; o >>= 1) {
                cl_join(px, ex, o, LPA);
                cl_join(py, ey, o, LPA);
                cl_join(pz, ez, o, LPA);
            }
            if (range_err) status_set(d.status, ST_RANGE);
            if (active && lane == 0) {
                float* f = fsum + 6 * g;
                f[0] = px; f[1] = ex; f[2] = py; f[3] = ey; f[4] = pz; f[5] = ez;
            }
        }
        // the next kick and drift touch only this CTA's own atoms: a block
        // barrier, no cluster barrier
        __syncthreads();
    }
    // every CTA has waited for all copies into its shared memory, so after
    // this barrier no copy reads a CTA's shared memory any more: all may exit
    cl.sync();
    if (owner && !ACCEL) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            s.x[3 * io + k] = x[k];
            s.v[3 * io + k] = v[k];
            s.a_old[3 * io + k] = a[k];
            d.xref[3 * io + k] = xref_s[3 * ko + k];
        }
    }
    // the lists for the next launch, if this one built them (with their own
    // reference positions: d.xref also serves the global lists, which other
    // calls rebuild)
    if (built) {
        for (int t = tid; t < 3 * na; t += CL_THREADS) xref_g[3 * (size_t)a0 + t] = xref_s[t];
        int4* dst4 = reinterpret_cast<int4*>(lst_g + (size_t)rank * per * cap);
        const int4* src4 = reinterpret_cast<const int4*>(lst);
#pragma unroll 4
        for (int t = tid; t < na * cap / 4; t += CL_THREADS) dst4[t] = src4[t];
        for (int t = tid; t < na; t += CL_THREADS) cnt_g[(size_t)rank * per + t] = cnt[t];
    }
    if (!ACCEL && rank == 0 && tid == 0) *since_g = since;
}

typedef void (*cluster_kernel_t)(Dev, StateView, double*, double, int, int, int, int, int*, int*, double*, int*, int, int64_t,
                                 int, int, double*, const double*, double*);

static cluster_kernel_t cluster_kernel(int lpa, bool accel = false)
{
    switch (lpa) {
    case 4: return accel ? k_cluster_vv<4, true> : k_cluster_vv<4, false>;
    case 8: return accel ? k_cluster_vv<8, true> : k_cluster_vv<8, false>;
    case 16: return accel ? k_cluster_vv<16, true> : k_cluster_vv<16, false>;
    default: return accel ? k_cluster_vv<32, true> : k_cluster_vv<32, false>;
    }
}

// Plan the cluster path for the current list capacity: cluster size (16 where
// the device allows it, else the portable 8), atoms per CTA, lanes per atom
// and shared-memory bytes. Returns false when the system does not qualify
// (one replica of a potential system under cubic boundaries, no
// thermostat, small enough for the shared-memory copies).
bool cluster_plan(nbg_ctx* c)
{
    c->cluster_ok = false;
    if (c->cluster_disabled || c->path != PATH_LIST || c->nrep != 1 || c->d.kind != NBG_SYSTEM_POTENTIAL ||
        c->d.bc != NBG_BC_CUBIC || c->d.therm != NBG_THERMO_NULL || c->baoab || c->n < 64 || c->n > 2048)
        return false;
    // (the cluster lists' rows are whole 16-byte units: cap rounded up to 4)
    const int n = (int)c->n, cap = (c->d.nbr_cap + 3) & ~3;
    for (int C = CL_MAX; C >= 8; C /= 2) {
        const int per = (n + C - 1) / C;
        if (per > 128) continue;  // owner threads: 4 warps x 32 lanes
        int lpa = 32;
        while (lpa > 4 && per * lpa > CL_THREADS) lpa /= 2;
        if (per * lpa > CL_THREADS) continue;
        const size_t bytes = sizeof(float4) * 4 * (size_t)n + sizeof(double) * (3 * (size_t)per + ((3 * per) & 1)) +
                             sizeof(int) * ((size_t)per * cap + per) + sizeof(float) * 6 * (size_t)per;
        if (bytes > 200 * 1024) continue;
        cluster_kernel_t k = cluster_kernel(lpa), ka = cluster_kernel(lpa, true);
        bool attrs_ok = true;
        for (cluster_kernel_t f : {k, ka}) {
            attrs_ok = attrs_ok &&
                       cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) == cudaSuccess &&
                       (C <= 8 || cudaFuncSetAttribute(f, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) ==
                                      cudaSuccess);
        }
        if (!attrs_ok) {
            cudaGetLastError();
            continue;
        }
        cudaLaunchConfig_t cfg = {};
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = C;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.gridDim = dim3(C);
        cfg.blockDim = dim3(CL_THREADS);
        cfg.dynamicSmemBytes = bytes;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        int clusters = 0;
        if (cudaOccupancyMaxActiveClusters(&clusters, (const void*)k, &cfg) != cudaSuccess || clusters < 1) {
            cudaGetLastError();
            continue;
        }
        c->cluster_ok = true;
        c->cluster_size = C;
        c->cluster_per = per;
        c->cluster_lpa = lpa;
        c->cluster_bytes = bytes;
        c->cluster_cap = cap;
        return true;
    }
    return false;
}

int launch_cluster_vv(nbg_ctx* c, const StateView& s, double dt, int64_t nsteps, int rebuild_every, int64_t step0,
                      unsigned* status)
{
    cluster_kernel_t k = cluster_kernel(c->cluster_lpa);
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = c->cluster_size;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(c->cluster_size);
    cfg.blockDim = dim3(CL_THREADS);
    cfg.dynamicSmemBytes = c->cluster_bytes;
    cfg.stream = c->stream;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    // a one-shot test of the timeout path (NBG_TEST_CLUSTER_DROP at context
    // creation): the launch drops the position copies of one step
    int drop = -2;
    if (c->cluster_test_drop != -2 && c->cluster_test_skip > 0) {
        --c->cluster_test_skip;
    } else if (c->cluster_test_drop != -2) {
        drop = c->cluster_test_drop < 0 ? (int)nsteps - 1 : std::min<int>(c->cluster_test_drop, (int)nsteps - 1);
        c->cluster_test_drop = -2;
    }
    Dev d = c->d;
    d.status = status;
    prof_begin(c);
    cudaError_t e = cudaLaunchKernelEx(&cfg, k, d, s, c->cluster_x, dt, (int)nsteps, rebuild_every,
                                       c->cluster_per, c->cluster_cap, c->cluster_lists, c->cluster_cnt,
                                       c->cluster_xref, c->cluster_since, c->cluster_lists_valid ? 1 : 0, step0,
                                       c->sink_on ? 1 : 0, drop, c->bk, (const double*)nullptr, (double*)nullptr);
    prof_end(c);
    if (e != cudaSuccess) return cuda_fail(c, e, "k_cluster_vv launch");
    NBG_LAUNCH_CHECK(c, "k_cluster_vv");
    return NBG_OK;
}

// The right-hand side of a small system (nbg_accel) as one cluster launch:
// positions from u, accelerations to dv (device addresses: pinned host
// memory mapped into the device's space, or device memory), the launch's
// own lists reused while no atom moved more than skin/2 from their build.
int launch_cluster_accel(nbg_ctx* c, const double* u, double* dv, unsigned* status)
{
    cluster_kernel_t k = cluster_kernel(c->cluster_lpa, true);
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = c->cluster_size;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(c->cluster_size);
    cfg.blockDim = dim3(CL_THREADS);
    cfg.dynamicSmemBytes = c->cluster_bytes;
    cfg.stream = c->stream;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    Dev d = c->d;
    d.status = status;
    prof_begin(c);
    cudaError_t e = cudaLaunchKernelEx(&cfg, k, d, c->st, c->cluster_x, 0.0, 1, 0, c->cluster_per, c->cluster_cap,
                                       c->cla_lists, c->cla_cnt, c->cla_xref, c->cluster_since,
                                       c->cla_valid ? 1 : 0, (int64_t)0, 0, -2, c->bk, u, dv);
    prof_end(c);
    if (e != cudaSuccess) return cuda_fail(c, e, "k_cluster_vv (right-hand side) launch");
    NBG_LAUNCH_CHECK(c, "k_cluster_vv");
    return NBG_OK;
}

// The launch floor of the cluster loop's shape: a kernel with the same CTAs,
// threads, shared memory and cluster that only passes one cluster barrier.
__global__ void __launch_bounds__(CL_THREADS, 1) k_cluster_empty(int* sink)
{
    extern __shared__ float4 ce_s[];
    cg::cluster_group cl = cg::this_cluster();
    if (threadIdx.x == 0) ce_s[0] = make_float4(0.f, 0.f, 0.f, 0.f);
    cl.sync();
    if (threadIdx.x == 0 && ce_s[0].x != 0.f) *sink = 1;  // never: keeps the store live
}

int cluster_launch_floor(nbg_ctx* c, double* us_single, double* us_per_launch)
{
    if (!c->cluster_ok) return NBG_ERR_UNSUPPORTED;
    if (cudaFuncSetAttribute(k_cluster_empty, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)c->cluster_bytes) !=
            cudaSuccess ||
        (c->cluster_size > 8 &&
         cudaFuncSetAttribute(k_cluster_empty, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess))
        return cuda_fail(c, cudaGetLastError(), "k_cluster_empty attributes");
    int* sink = nullptr;
    if (cudaMalloc(&sink, sizeof(int)) != cudaSuccess) return cuda_fail(c, cudaGetLastError(), "probe sink");
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = c->cluster_size;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(c->cluster_size);
    cfg.blockDim = dim3(CL_THREADS);
    cfg.dynamicSmemBytes = c->cluster_bytes;
    cfg.stream = c->stream;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < 20 && e == cudaSuccess; ++k) e = cudaLaunchKernelEx(&cfg, k_cluster_empty, sink);
    const int reps = 200;
    float ms = 0.f, single = 0.f;
    if (e == cudaSuccess) {
        // back to back
        cudaEventRecord(e0, c->stream);
        for (int k = 0; k < reps && e == cudaSuccess; ++k) e = cudaLaunchKernelEx(&cfg, k_cluster_empty, sink);
        cudaEventRecord(e1, c->stream);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    }
    // one at a time, the host waiting for each
    for (int k = 0; k < reps && e == cudaSuccess; ++k) {
        float m1 = 0.f;
        cudaEventRecord(e0, c->stream);
        e = cudaLaunchKernelEx(&cfg, k_cluster_empty, sink);
        cudaEventRecord(e1, c->stream);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&m1, e0, e1);
        single += m1;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    if (e != cudaSuccess) return cuda_fail(c, e, "cluster launch floor");
    if (us_per_launch) *us_per_launch = 1e3 * ms / reps;
    if (us_single) *us_single = 1e3 * single / reps;
    return NBG_OK;
}

