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
//   k_cell_fill  : atom -> cell by its wrapped position, slot by atomicAdd
//   k_cell_sort  : each cell's atoms sorted by index (deterministic lists),
//                  counts moved to cell_n and cleared for the next build
//   k_list_build : 27-cell scan per atom; the list is column-major
//                  (nbr[k*n + i]) for thread-per-atom force kernels and
//                  row-major (nbr[i*cap + k]) for lanes-per-atom kernels
#include "nbg_internal.cuh"

struct ListCtl {
    StepRef pos;  // time index of the positions: its parity picks the rebuild_flag word
    int force;    // host-forced rebuild
};

__device__ __forceinline__ int read_parity(const ListCtl& L) { return (int)(step_of(L.pos) & 1); }

__device__ __forceinline__ bool need_build(const Dev& d, const ListCtl& L)
{
    return L.force || d.rebuild_flag[read_parity(L)] != 0;
}

__device__ __forceinline__ int cell_coord(float h, const RepDev& R)
{
    int c = (int)floorf(h * (float)R.cell_inv);
    if (c < 0) c = 0;
    if (c >= R.nc) c = R.nc - 1;
    return c;
}

__global__ void k_cell_fill(Dev d, ListCtl L)
{
    if (!need_build(d, L)) return;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < d.n; i += (int64_t)gridDim.x * blockDim.x) {
        const RepDev& R = d.reps[d.rep_of[i]];
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
    if (!need_build(d, L)) return;
    extern __shared__ int sh[];
    for (int cell = blockIdx.x; cell < d.ncell_total; cell += gridDim.x) {
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

__global__ void k_list_build(Dev d, ListCtl L, const double* X)
{
    if (blockIdx.x == 0 && threadIdx.x == 0) d.rebuild_flag[read_parity(L) ^ 1] = 0;
    if (!need_build(d, L)) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(d.build_count, 1ull);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < d.n; i += (int64_t)gridDim.x * blockDim.x) {
        const RepDev& R = d.reps[d.rep_of[i]];
        float4 hi = d.phi[i], lo = d.plo[i];
        int cx = cell_coord(hi.x, R), cy = cell_coord(hi.y, R), cz = cell_coord(hi.z, R);
        int cnt = 0;
        const bool water = d.kind == NBG_SYSTEM_WATER;
        const int o0 = R.nc >= 3 ? -1 : 0, o1 = R.nc >= 3 ? 1 : 0;
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
                        int j = atoms[k];
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
    if (blockIdx.x == 0 && threadIdx.x == 0) d.rebuild_flag[read_parity(L) ^ 1] = 0;
    if (!need_build(d, L)) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(d.build_count, 1ull);
    const int lane = threadIdx.x % LPA;
    const int gbase = (threadIdx.x % 32) - lane;  // first lane of the group within the warp
    const unsigned gmask = (LPA == 32) ? 0xffffffffu : (((1u << LPA) - 1u) << gbase);
    const int64_t i = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / LPA;
    if (i >= d.n) return;  // whole groups leave together
    const RepDev& R = d.reps[d.rep_of[i]];
    const float4 hi = d.phi[i], lo = d.plo[i];
    const int cx = cell_coord(hi.x, R), cy = cell_coord(hi.y, R), cz = cell_coord(hi.z, R);
    const bool water = d.kind == NBG_SYSTEM_WATER;
    int cnt = 0;
    int* out = d.nbr + i * d.nbr_istride;
    const int o0 = R.nc >= 3 ? -1 : 0, o1 = R.nc >= 3 ? 1 : 0;
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
                        j = atoms[k];
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

int launch_list_build(nbg_ctx* c, const StateView& s, bool force, StepRef pos)
{
    ListCtl L{pos, force ? 1 : 0};
    k_cell_fill<<<grid_for(c->n, 256), 256, 0, c->stream>>>(c->d, L);
    NBG_LAUNCH_CHECK(c, "k_cell_fill");
    int cells = c->d.ncell_total;
    int gs = cells < 65536 ? cells : 65536;
    k_cell_sort<<<gs, 128, sizeof(int) * c->d.cell_cap, c->stream>>>(c->d, L);
    NBG_LAUNCH_CHECK(c, "k_cell_sort");
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
    NBG_LAUNCH_CHECK(c, "k_list_build");
    return NBG_OK;
}
