// k_lists.cu - cell lists and Verlet lists under cubic periodic boundaries.
//
// The reference evaluates every ordered pair (O(N^2), basic_potentials.jl:
// 253-267, 288-299); these lists only restrict the candidates. A Verlet list
// holds every j with FP32 r^2 < (cutoff + skin)^2 (inflated), so as long as no
// atom moved more than skin/2 since the build it is a superset of the
// reference's pair set; the force kernels then apply the exact test.
//
// Build, skipped on device unless a rebuild is due (host-forced every
// rebuild_every steps, or an atom moved more than skin/2):
//   k_cell_fill        : atom -> cell by its wrapped position (the image taken
//                        at the build is kept for the packing until the
//                        next), slot by atomicAdd
//   k_cell_sort        : each cell's atoms sorted by index (deterministic
//                        lists), counts moved to cell_n and cleared for the
//                        next build
//   k_list_build_warps : (at least two cells per SM) one warp per 32 atoms of a cell; the
//                        stencil cells' atoms (split-position hi parts moved
//                        by the periodic shift into the cell's frame) pass
//                        through a per-warp buffer in scan order and every
//                        atom of the cell tests them with broadcast reads. The
//                        list is column-major (nbr[k*n + i]) for
//                        thread-per-atom force kernels and row-major
//                        (nbr[i*cap + k]) for lanes-per-atom kernels.
//   k_list_build(_lanes): (fewer cells) a thread or a group of lanes per atom
//                        scanning its 27 cells with gathers of the split positions.
#include "nbg_internal.cuh"

struct ListCtl {
    StepRef pos;  // time index of the positions: its parity picks the rebuild_flag word
    int force;    // host-forced rebuild
};

__device__ __forceinline__ int read_parity(const ListCtl& L) { return (int)(step_of(L.pos) & 1); }

// Replica r's list is rebuilt when the host forces it or one of its atoms
// moved more than skin/2 (flags per replica, so one fast atom in a batch
// rebuilds only its own replica).
__device__ __forceinline__ bool need_build(const Dev& d, const ListCtl& L, int rep)
{
    return L.force || d.rebuild_flag[read_parity(L) * d.nrep + rep] != 0;
}

__device__ __forceinline__ int cell_coord(float h, const RepDev& R)
{
    int c = (int)floorf(h * (float)R.cell_inv);
    if (c < 0) c = 0;
    if (c >= R.nc) c = R.nc - 1;
    return c;
}

// At a build the atom's periodic image is taken afresh (the wrap into
// [0, L)), stored in d.img and its split position packed with it; until the
// next build the drift packs with that image, so that a replica's lists and
// positions keep one frame.
__global__ void k_cell_fill(Dev d, ListCtl L, const double* X)
{
    // the other parity's flags start clean for the next drift (nothing of
    // this rebuild reads them)
    const int other = (read_parity(L) ^ 1) * d.nrep;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < d.nrep; r += gridDim.x * blockDim.x)
        d.rebuild_flag[other + r] = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < d.n; i += (int64_t)gridDim.x * blockDim.x) {
        if (!need_build(d, L, d.rep_of[i])) continue;
        const RepDev& R = d.reps[d.rep_of[i]];
        if (d.img && d.bc == NBG_BC_CUBIC) {
            double im[3];
            for (int k = 0; k < 3; ++k) {
                const double p = X[3 * i + k];
                double m = floor(p * R.invL);
                const double w = fma(-R.L, m, p);
                if (w < 0.0) m -= 1.0;
                else if (w >= R.L) m += 1.0;
                im[k] = m;
                d.img[3 * i + k] = m;
            }
            const double p[3] = {X[3 * i], X[3 * i + 1], X[3 * i + 2]};
            float hh[3], ll[3];
            split_position_image(R, p, im, hh, ll);
            d.phi[i] = make_float4(hh[0], hh[1], hh[2], d.phi[i].w);
            d.plo[i] = make_float4(ll[0], ll[1], ll[2], d.plo[i].w);
        }
        float4 h = d.phi[i];
        int cx = cell_coord(h.x, R), cy = cell_coord(h.y, R), cz = cell_coord(h.z, R);
        int cell = R.cell0 + (cx * R.nc + cy) * R.nc + cz;
        int slot = atomicAdd(&d.cell_count[cell], 1);
        if (slot < d.cell_cap) d.cell_atoms[(int64_t)cell * d.cell_cap + slot] = (int)i;
        else status_set(d.status, ST_CELL_OVERFLOW);
    }
}

// One block per cell: rank sort of the (distinct) atom indices.
__global__ void k_cell_sort(Dev d, ListCtl L)
{
    extern __shared__ int sh[];
    for (int cell = blockIdx.x; cell < d.ncell_total; cell += gridDim.x) {
        const int rep = d.cell_rep[cell];
        if (!need_build(d, L, rep)) continue;
        if (threadIdx.x == 0 && cell == d.reps[rep].cell0) atomicAdd(d.build_count, 1ull);  // one per replica
        int cnt = d.cell_count[cell];
        if (cnt > d.cell_cap) cnt = d.cell_cap;
        int* src = d.cell_atoms + (int64_t)cell * d.cell_cap;
        for (int k = threadIdx.x; k < cnt; k += blockDim.x) sh[k] = src[k];
        __syncthreads();
        for (int k = threadIdx.x; k < cnt; k += blockDim.x) {
            int v = sh[k];
            int rank = 0;
            for (int m = 0; m < cnt; ++m) rank += (sh[m] < v);
            src[rank] = v;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            d.cell_n[cell] = cnt;
            d.cell_count[cell] = 0;
        }
        __syncthreads();
    }
}

// Per-atom builds, for systems with too few cells to fill the GPU one
// warp per cell: the thread (or group of LPA lanes) of an atom scans its
// 27 cells in the same order as the warp-per-cell build.
__global__ void k_list_build(Dev d, ListCtl L, const double* X)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < d.n; i += (int64_t)gridDim.x * blockDim.x) {
        if (!need_build(d, L, d.rep_of[i])) continue;
        const RepDev& R = d.reps[d.rep_of[i]];
        float4 hi = d.phi[i], lo = d.plo[i];
        int cx = cell_coord(hi.x, R), cy = cell_coord(hi.y, R), cz = cell_coord(hi.z, R);
        int cnt = 0;
        const bool water = d.kind == NBG_SYSTEM_WATER;
        const int o0 = -R.ns, o1 = R.ns;
        for (int ox = o0; ox <= o1; ++ox) {
            int nx = cx + ox;
            nx += (nx < 0) ? R.nc : 0;
            nx -= (nx >= R.nc) ? R.nc : 0;
            for (int oy = o0; oy <= o1; ++oy) {
                int ny = cy + oy;
                ny += (ny < 0) ? R.nc : 0;
                ny -= (ny >= R.nc) ? R.nc : 0;
                for (int oz = o0; oz <= o1; ++oz) {
                    int nz = cz + oz;
                    nz += (nz < 0) ? R.nc : 0;
                    nz -= (nz >= R.nc) ? R.nc : 0;
                    int cell = R.cell0 + (nx * R.nc + ny) * R.nc + nz;
                    int m = d.cell_n[cell];
                    const int* atoms = d.cell_atoms + (int64_t)cell * d.cell_cap;
                    for (int k = 0; k < m; ++k) {
                        int j = dbg_index(atoms[k], d.n, (int)i, d.status);
                        if (j == (int)i) continue;
                        if (water && (j / 3 == (int)(i / 3))) continue;  // intramolecular: never a pair
                        float4 hj = d.phi[j], lj = d.plo[j];
                        float3 dr = split_diff(hi, lo, hj, lj, true, R);
                        float r2 = dr.x * dr.x + dr.y * dr.y + dr.z * dr.z;
                        if (r2 < R.rl2) {
                            if (cnt < d.nbr_cap) d.nbr[(int64_t)cnt * d.nbr_kstride + i * d.nbr_istride] = j;
                            ++cnt;
                        }
                    }
                }
            }
        }
        if (cnt > d.nbr_cap) {
            status_set(d.status, ST_NBR_OVERFLOW);
            cnt = d.nbr_cap;
        }
        d.nbr_count[i] = cnt;
        d.xref[3 * i] = X[3 * i];
        d.xref[3 * i + 1] = X[3 * i + 1];
        d.xref[3 * i + 2] = X[3 * i + 2];
    }
}

// LPA lanes per atom: the group scans the 27 cells in the same order, each
// chunk of LPA consecutive cell entries tested in parallel; accepted entries
// keep their scan order through a ballot prefix count, so the row-major list
// is identical to the one-thread-per-atom list.
template <int LPA>
__global__ void __launch_bounds__(256) k_list_build_lanes(Dev d, ListCtl L, const double* X)
{
    const int lane = threadIdx.x % LPA;
    const int gbase = (threadIdx.x % 32) - lane;  // first lane of the group within the warp
    const unsigned gmask = (LPA == 32) ? 0xffffffffu : (((1u << LPA) - 1u) << gbase);
    const int64_t i = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / LPA;
    if (i >= d.n) return;  // whole groups leave together
    if (!need_build(d, L, d.rep_of[i])) return;
    const RepDev& R = d.reps[d.rep_of[i]];
    const float4 hi = d.phi[i], lo = d.plo[i];
    const int cx = cell_coord(hi.x, R), cy = cell_coord(hi.y, R), cz = cell_coord(hi.z, R);
    const bool water = d.kind == NBG_SYSTEM_WATER;
    int cnt = 0;
    int* out = d.nbr + i * d.nbr_istride;
    const int o0 = -R.ns, o1 = R.ns;
    for (int ox = o0; ox <= o1; ++ox) {
        int nx = cx + ox;
        nx += (nx < 0) ? R.nc : 0;
        nx -= (nx >= R.nc) ? R.nc : 0;
        for (int oy = o0; oy <= o1; ++oy) {
            int ny = cy + oy;
            ny += (ny < 0) ? R.nc : 0;
            ny -= (ny >= R.nc) ? R.nc : 0;
            for (int oz = o0; oz <= o1; ++oz) {
                int nz = cz + oz;
                nz += (nz < 0) ? R.nc : 0;
                nz -= (nz >= R.nc) ? R.nc : 0;
                const int cell = R.cell0 + (nx * R.nc + ny) * R.nc + nz;
                const int m = d.cell_n[cell];
                const int* atoms = d.cell_atoms + (int64_t)cell * d.cell_cap;
                for (int k0 = 0; k0 < m; k0 += LPA) {
                    const int k = k0 + lane;
                    bool take = false;
                    int j = 0;
                    if (k < m) {
                        j = dbg_index(atoms[k], d.n, (int)i, d.status);
                        if (j != (int)i && !(water && (j / 3 == (int)(i / 3)))) {
                            float3 dr = split_diff(hi, lo, d.phi[j], d.plo[j], true, R);
                            float r2 = dr.x * dr.x + dr.y * dr.y + dr.z * dr.z;
                            take = r2 < R.rl2;
                        }
                    }
                    const unsigned bal = __ballot_sync(gmask, take);
                    if (take) {
                        const int pos = cnt + __popc(bal & gmask & ((1u << (gbase + lane)) - 1u));
                        if (pos < d.nbr_cap) out[pos] = j;
                    }
                    cnt += __popc(bal & gmask);
                }
            }
        }
    }
    if (lane == 0) {
        if (cnt > d.nbr_cap) {
            status_set(d.status, ST_NBR_OVERFLOW);
            cnt = d.nbr_cap;
        }
        d.nbr_count[i] = cnt;
    }
    if (lane < 3) d.xref[3 * i + lane] = X[3 * i + lane];
}

// Warp per (cell, chunk of 32 of its atoms): lane l holds atom l of the
// chunk. The stencil's cells (125 or 27, or for a one-cell replica 1)
// pass their atoms through a per-warp buffer of 32 candidates (split-position
// hi parts moved by the periodic shift into the cell's frame, index in w) read
// back by broadcast; the next chunk's index and position gathers are issued
// before the current chunk's tests. The test r^2 < rl2 on the hi parts is the
// list's superset test (the force kernels classify every pair exactly). The
// candidates come in the stencil order of the per-atom builders (cell q =
// ((ox+ns) w + oy+ns) w + oz+ns, then slot order), so the lists are the same.
#define LW_WARPS 4
#define LW_NB 125

template <bool ONE, bool WATER>
__device__ __forceinline__ int lw_test(const float4* cand, int bn, const float4& hi, int i, int mol0, float rl2,
                                       const RepDev& R, int* row, int64_t kstride, int cap, int lcnt)
{
#pragma unroll 4
    for (int k = 0; k < bn; ++k) {
        const float4 c = cand[k];
        float dx = c.x - hi.x, dy = c.y - hi.y, dz = c.z - hi.z;
        if (ONE) {
            // s = rint(d / L) by the 1.5 * 2^23 trick (|d / L| <= 1)
            const float magic = 12582912.0f;
            dx = __fmaf_rn(-__fsub_rn(__fmaf_rn(dx, R.invLf, magic), magic), R.Lh, dx);
            dy = __fmaf_rn(-__fsub_rn(__fmaf_rn(dy, R.invLf, magic), magic), R.Lh, dy);
            dz = __fmaf_rn(-__fsub_rn(__fmaf_rn(dz, R.invLf, magic), magic), R.Lh, dz);
        }
        const float r2 = dx * dx + dy * dy + dz * dz;
        const int j = __float_as_int(c.w);
        if (r2 < rl2 && j != i && (!WATER || (unsigned)(j - mol0) >= 3u)) {
            if (lcnt < cap) row[(int64_t)lcnt * kstride] = j;
            ++lcnt;
        }
    }
    return lcnt;
}

__global__ void __launch_bounds__(LW_WARPS * 32) k_list_build_warps(Dev d, ListCtl L, const double* X, int chunks)
{
    __shared__ int nb_code[LW_WARPS][LW_NB];  // stencil cell | (shift + 1) per axis in bits 24-29
    __shared__ int nb_cnt[LW_WARPS][LW_NB];
    __shared__ float4 cand[LW_WARPS][32];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const bool water = d.kind == NBG_SYSTEM_WATER;
    // work item: (cell, c), c < chunks; it takes the cell's atoms from 32 c
    // in strides of 32 chunks, so that cells holding many atoms spread over
    // several warps
    const int64_t items = (int64_t)d.ncell_total * chunks;
    for (int64_t it = blockIdx.x * (int64_t)LW_WARPS + wid; it < items; it += (int64_t)gridDim.x * LW_WARPS) {
        const int cell = (int)(it / chunks);
        const int c0 = (int)(it % chunks) * 32;
        const int rep = d.cell_rep[cell];
        if (!need_build(d, L, rep)) continue;
        const int cnt = min(d.cell_n[cell], d.cell_cap);
        if (c0 >= cnt) continue;
        const RepDev& R = d.reps[rep];
        const int nc = R.nc;
        const int lc = cell - R.cell0;
        const int cx = lc / (nc * nc), cy = (lc / nc) % nc, cz = lc % nc;
        const bool one = R.ns == 0;  // one cell holds the replica: minimum image per pair
        const int w = 2 * R.ns + 1;  // stencil width (1, 3 or 5)
        const int nnb = w * w * w;
        __syncwarp();  // the previous cell's tables are consumed
        for (int q = lane; q < nnb; q += 32) {
            const int ox = q / (w * w) - R.ns, oy = (q / w) % w - R.ns, oz = q % w - R.ns;
            int nx = cx + ox, ny = cy + oy, nz = cz + oz;
            int sx = 1, sy = 1, sz = 1;
            if (nx < 0) { nx += nc; sx = 0; }
            if (nx >= nc) { nx -= nc; sx = 2; }
            if (ny < 0) { ny += nc; sy = 0; }
            if (ny >= nc) { ny -= nc; sy = 2; }
            if (nz < 0) { nz += nc; sz = 0; }
            if (nz >= nc) { nz -= nc; sz = 2; }
            const int cq = R.cell0 + (nx * nc + ny) * nc + nz;
            nb_code[wid][q] = cq | (sx << 24) | (sy << 26) | (sz << 28);
            nb_cnt[wid][q] = min(d.cell_n[cq], d.cell_cap);
        }
        __syncwarp();
        const float Lh = R.Lh, rl2 = R.rl2;
        const int* atoms = d.cell_atoms + (int64_t)cell * d.cell_cap;
        for (int a0 = c0; a0 < cnt; a0 += 32 * chunks) {
            const int a = a0 + lane;
#ifdef NBG_DEBUG
            const int i_read = a < cnt ? atoms[a] : -1;
            const bool active = a < cnt && dbg_index(i_read, d.n, -1, d.status) >= 0;
            const int i = active ? i_read : -1;
#else
            const bool active = a < cnt;
            const int i = active ? atoms[a] : -1;
#endif
            const float4 hi = active ? d.phi[i] : make_float4(0.f, 0.f, 0.f, 0.f);
            const int mol0 = water && active ? 3 * (i / 3) : -8;  // first atom of i's molecule
            int* row = d.nbr + (int64_t)(active ? i : 0) * d.nbr_istride;
            int lcnt = 0;
            // chunk (q, b0): atoms b0 .. b0 + 31 of stencil cell q
            int q = 0;
            while (q < nnb && nb_cnt[wid][q] == 0) ++q;
            int b0 = 0;
            int jn = -1;
            float4 hn = make_float4(0.f, 0.f, 0.f, 0.f);
            if (q < nnb) {
                const int cq = nb_code[wid][q] & 0xffffff;
                if (lane < nb_cnt[wid][q]) {
                    jn = dbg_index(d.cell_atoms[(int64_t)cq * d.cell_cap + lane], d.n, 0, d.status);
                    hn = d.phi[jn];
                }
            }
            while (q < nnb) {
                const int code = nb_code[wid][q];
                const int cn = nb_cnt[wid][q];
                const int bn = min(32, cn - b0);
                const int j = jn;
                const float4 hj = hn;
                // the next chunk's gathers go out before this chunk's tests
                int q2 = q, b2 = b0 + 32;
                if (b2 >= cn) {
                    b2 = 0;
                    ++q2;
                    while (q2 < nnb && nb_cnt[wid][q2] == 0) ++q2;
                }
                if (q2 < nnb) {
                    const int cq2 = nb_code[wid][q2] & 0xffffff;
                    jn = -1;
                    if (b2 + lane < nb_cnt[wid][q2]) {
                        jn = dbg_index(d.cell_atoms[(int64_t)cq2 * d.cell_cap + b2 + lane], d.n, 0, d.status);
                        hn = d.phi[jn];
                    }
                }
                const float sx = (float)(((code >> 24) & 3) - 1) * Lh;
                const float sy = (float)(((code >> 26) & 3) - 1) * Lh;
                const float sz = (float)(((code >> 28) & 3) - 1) * Lh;
                if (lane < bn) cand[wid][lane] = make_float4(hj.x + sx, hj.y + sy, hj.z + sz, __int_as_float(j));
                __syncwarp();
                if (active) {
                    if (one)
                        lcnt = water ? lw_test<true, true>(cand[wid], bn, hi, i, mol0, rl2, R, row, d.nbr_kstride, d.nbr_cap, lcnt)
                                     : lw_test<true, false>(cand[wid], bn, hi, i, mol0, rl2, R, row, d.nbr_kstride, d.nbr_cap, lcnt);
                    else
                        lcnt = water ? lw_test<false, true>(cand[wid], bn, hi, i, mol0, rl2, R, row, d.nbr_kstride, d.nbr_cap, lcnt)
                                     : lw_test<false, false>(cand[wid], bn, hi, i, mol0, rl2, R, row, d.nbr_kstride, d.nbr_cap, lcnt);
                }
                __syncwarp();
                q = q2;
                b0 = b2;
            }
            if (active) {
                if (lcnt > d.nbr_cap) {
                    status_set(d.status, ST_NBR_OVERFLOW);
                    lcnt = d.nbr_cap;
                }
                d.nbr_count[i] = lcnt;
                d.xref[3 * i] = X[3 * i];
                d.xref[3 * i + 1] = X[3 * i + 1];
                d.xref[3 * i + 2] = X[3 * i + 2];
            }
        }
    }
}

#ifdef NBG_DEBUG
// Debug builds only: entry 0 of atom 0's Verlet-list row (nbr[0] in both
// layouts) becomes n + k, an index past every per-atom buffer, so that the
// tests see the list readers' index checks report it (NBG_ERR_INDEX).
__global__ void k_plant_index(Dev d, int k)
{
    if (threadIdx.x == 0 && blockIdx.x == 0 && d.nbr_count[0] > 0) d.nbr[0] = (int)(d.n + k);
}

int launch_plant_index(nbg_ctx* c, int k)
{
    k_plant_index<<<1, 32, 0, c->stream>>>(c->d, k);
    NBG_LAUNCH_CHECK(c, "k_plant_index");
    return NBG_OK;
}
#endif

int launch_list_build(nbg_ctx* c, const StateView& s, bool force, StepRef pos)
{
    NBG_RANGE("launch_list_build");
    c->accel_lists_valid = false;  // the lists follow other positions now
    c->ens_lists_valid = false;
    ListCtl L{pos, force ? 1 : 0};
    // The kernels run at every step of a captured graph and skip the atoms
    // and cells of replicas without a due rebuild. The fill and the sort
    // loop over their items on a few waves of blocks, so that a step with no
    // rebuild (or, in a batch, few) does not schedule a block per cell; the
    // list build keeps a warp per item, whose work is too uneven for a
    // fixed share per warp.
    const int64_t wave = (int64_t)c->sms * 8;
    k_cell_fill<<<(unsigned)std::min<int64_t>(grid_for(c->n, 256), wave), 256, 0, c->stream>>>(c->d, L, s.x);
    NBG_LAUNCH_CHECK(c, "k_cell_fill");
    const int64_t cells = c->d.ncell_total;
    k_cell_sort<<<(unsigned)std::min<int64_t>(cells, 4 * wave), 128, sizeof(int) * c->d.cell_cap, c->stream>>>(c->d, L);
    NBG_LAUNCH_CHECK(c, "k_cell_sort");
    if (c->d.ncell_total >= 2 * c->sms) {
        // warps per cell from the mean occupancy (with margin); fuller cells loop
        const double occ = (double)c->n / std::max(c->d.ncell_total, 1);
        const int chunks = std::max(1, std::min((c->d.cell_cap + 31) / 32, (int)std::ceil(1.5 * occ / 32.0)));
        const int64_t items = (int64_t)c->d.ncell_total * chunks;
        const int64_t blocks = std::min<int64_t>((items + LW_WARPS - 1) / LW_WARPS, 1 << 20);
        k_list_build_warps<<<(unsigned)blocks, LW_WARPS * 32, 0, c->stream>>>(c->d, L, s.x, chunks);
    } else {
        const int lpa = c->list_lpa;
        if (lpa <= 1) {
            k_list_build<<<grid_for(c->n, 128), 128, 0, c->stream>>>(c->d, L, s.x);
        } else {
            const int per_block = 256 / lpa;
            const int grid = (int)((c->n + per_block - 1) / per_block);
            if (lpa == 4) k_list_build_lanes<4><<<grid, 256, 0, c->stream>>>(c->d, L, s.x);
            else if (lpa == 8) k_list_build_lanes<8><<<grid, 256, 0, c->stream>>>(c->d, L, s.x);
            else if (lpa == 16) k_list_build_lanes<16><<<grid, 256, 0, c->stream>>>(c->d, L, s.x);
            else k_list_build_lanes<32><<<grid, 256, 0, c->stream>>>(c->d, L, s.x);
        }
    }
    NBG_LAUNCH_CHECK(c, "k_list_build");
    return NBG_OK;
}
