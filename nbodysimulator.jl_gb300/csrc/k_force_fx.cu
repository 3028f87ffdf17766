// k_force_fx.cu - the Verlet-list pair forces (Lennard-Jones and reaction-
// field electrostatics, basic_potentials.jl:240-304) on fixed-point box
// coordinates, with the neighbour lists staged into shared memory by the
// tensor memory accelerator.
//
// Positions: q = x / L * 2^32 modulo 2^32 per component (uint32, written by
// the drift from the FP64 state). The wrapping 32-bit difference q_i - q_j,
// read as int32, is the minimum image of x_i - x_j in units u = L / 2^32,
// mapped into [-L/2, L/2) as the reference's while loops do
// (boundary_conditions.jl:138-165); one int-to-float conversion rounds it to
// 2^-24 of |r_ij| (the split hi/lo form's accuracy) and the positions carry
// 2^-32 of the box. One 16-byte record (x, y, z, charge) per neighbour is
// gathered instead of two, and no per-pair image arithmetic is left.
//
// Exact pair set: FP32 r^2 (box units) decides the clear cases; a pair
// within CLASSIFY_MARGIN of a cutoff, or beyond the half-box band where the
// image could differ, is decided again in the reference's FP64 arithmetic on
// the unwrapped positions (pair_fallback), as in the split form.
//
// Lists: row-major, nbr[i * cap + k]. A block owns tiles of A = 256 / LPA
// consecutive atoms in turn (a persistent grid). For the next tile, one warp
// reads the atoms' counts and one thread issues cp.async.bulk.tensor copies
// of the needed 32-entry column boxes ([A rows] x [128 B], 128-byte swizzle)
// into the other of two shared-memory stages, completing on that stage's
// mbarrier; the block meanwhile computes the current tile from its stage.
// LPA lanes per atom take two entries per iteration (packed FP32x2 for the
// arithmetic), keep FP32 partials, and join them by the compensated
// butterfly of the split-form kernel; one FP64 multiply by 1/m per component.
#include <cuda.h>
#include <cudaTypedefs.h>

#include "fx_pair.cuh"

#define FX_THREADS 256
#define FX_WAIT_TRIES (1u << 24)

__device__ __forceinline__ unsigned fx_smem(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void fx_mbar_init(unsigned a, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(count) : "memory");
}

__device__ __forceinline__ void fx_mbar_expect(unsigned a, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(a), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool fx_mbar_try(unsigned a, unsigned parity)
{
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    return ok != 0;
}

// One [rows] x [32 entries] box of the list into shared memory at dst
// (1024-byte aligned), completing on mbar.
__device__ __forceinline__ void fx_tma_box(unsigned dst, const CUtensorMap* map, int col, int row, unsigned mbar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
            "r"(dst),
        "l"(map), "r"(col), "r"(row), "r"(mbar)
        : "memory");
}

// Entry k of row a of a stage: box k / 32; within the box's 128-byte row the
// 16-byte chunk index is swizzled by the row (the 128-byte swizzle pattern).
__device__ __forceinline__ int fx_entry(const unsigned char* stage, int A, int a, int k)
{
    const int b = k >> 5, c = k & 31;
    const int off = b * A * 128 + a * 128 + ((((c >> 2) ^ (a & 7))) << 4) + ((c & 3) << 2);
    return *reinterpret_cast<const int*>(stage + off);
}


template <int LPA, int POT>
__global__ void __launch_bounds__(FX_THREADS) k_force_fx(Dev d, StateView s, const __grid_constant__ CUtensorMap map,
                                                         int nbox_cap)
{
    constexpr int A = FX_THREADS / LPA;  // atoms per tile
    constexpr bool HAS_LJ = POT == FX_LJ || POT == FX_LJEL || POT == FX_WATER;
    constexpr bool HAS_EL = POT == FX_EL || POT == FX_LJEL || POT == FX_WATER;
    __shared__ __align__(8) unsigned long long mbar[2];
    __shared__ int s_nbox[2];
    extern __shared__ unsigned char fx_dyn[];
    const int tid = threadIdx.x, lane = tid % LPA, a = tid / LPA;
    const unsigned dyn = fx_smem(fx_dyn);
    const unsigned base = (dyn + 1023u) & ~1023u;
    const unsigned stage_bytes = (unsigned)nbox_cap * A * 128u;
    unsigned char* const stage0 = fx_dyn + (base - dyn);  // stage st at stage0 + st * stage_bytes
    const int64_t ntiles = (d.n + A - 1) / A;
    if (tid == 0) {
        fx_mbar_init(fx_smem(&mbar[0]), 1);
        fx_mbar_init(fx_smem(&mbar[1]), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    // warp 0: the tile's largest count sets how many column boxes to copy
    auto issue = [&](int64_t t, int st) {
        int mx = 0;
        for (int r = tid; r < A; r += 32) {
            const int64_t i = t * A + r;
            if (i < d.n) mx = max(mx, min(d.nbr_count[i], d.nbr_cap));
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        const int nb = min((mx + 31) >> 5, nbox_cap);
        if (tid == 0) {
            s_nbox[st] = nb;
            const unsigned mb = fx_smem(&mbar[st]);
            if (nb == 0) {
                asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(mb) : "memory");
            } else {
                // the stage's previous contents were read by generic loads
                // (ordered by the block barrier before this call)
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                fx_mbar_expect(mb, (unsigned)nb * A * 128u);
                const unsigned dst = base + (unsigned)st * stage_bytes;
                for (int b = 0; b < nb; ++b) fx_tma_box(dst + (unsigned)b * A * 128u, &map, b * 32, (int)(t * A), mb);
            }
        }
    };

    bool range_err = false, timeout = false;
    int pend0 = -1, pend1 = -1;  // parities of copies still in flight at a timeout (stages 0, 1)
    int it = 0;
    if (blockIdx.x < ntiles && tid < 32) issue(blockIdx.x, 0);
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x, ++it) {
        const int st = it & 1;
        const int64_t tn = t + gridDim.x;
        if (tn < ntiles && tid < 32) issue(tn, st ^ 1);
        // the current stage (bounded wait: a copy of valid memory completes);
        // the block agrees on a timeout before anyone leaves the loop
        const unsigned mb = fx_smem(&mbar[st]);
        const unsigned parity = (unsigned)((it >> 1) & 1);
        unsigned tries = 0;
        bool late = false;
        while (!fx_mbar_try(mb, parity)) {
            if (++tries > FX_WAIT_TRIES) {
                late = true;
                break;
            }
        }
        if (__syncthreads_or(late)) {
            timeout = true;
            // copies in flight: this tile's stage, and the next tile's
            const int pn = tn < ntiles ? (int)(((it + 1) >> 1) & 1) : -1;
            pend0 = st == 0 ? (int)parity : pn;
            pend1 = st == 0 ? pn : (int)parity;
            break;
        }

        const unsigned char* stage = stage0 + (unsigned)st * stage_bytes;
        const int64_t i = t * A + a;
        const bool active = i < d.n;
        const int64_t ia = active ? i : 0;
        const RepDev& R = d.reps[d.rep_of[ia]];
        const uint4 qi = d.pfx[ia];
        const int cnt = active ? min(min(d.nbr_count[ia], d.nbr_cap), s_nbox[st] * 32) : 0;
        const bool lj_i = HAS_LJ && (POT != FX_WATER || (ia % 3) == 0);
        // k q_i / (u^2 fscale): rinv^3 in box units times this is the
        // electrostatic factor in the units of the LJ sum
        const float kqi = HAS_EL ? (float)(d.charge[ia] * R.fx_kq) : 0.0f;
        const float lj_lo = R.fx_lj_lo, lj_hi = R.fx_lj_hi, el_lo = R.fx_el_lo, el_hi = R.fx_el_hi;
        const float sig2h = R.fx_sig2_hi, sig2l = R.fx_sig2_lo, krf = R.fx_krf;
        float2 px = make_float2(0.f, 0.f), py = px, pz = px;
        // the next iteration's entries and gathers are issued before this
        // iteration's arithmetic (two neighbours ahead per lane)
        int jn0 = 0, jn1 = 0;
        uint4 qn0 = qi, qn1 = qi;
        if (lane < cnt) {
            jn0 = dbg_index(fx_entry(stage, A, a, lane), d.n, (int)ia, d.status);
            jn1 = lane + LPA < cnt ? dbg_index(fx_entry(stage, A, a, lane + LPA), d.n, (int)ia, d.status) : jn0;
            qn0 = __ldg(&d.pfx[jn0]);
            qn1 = __ldg(&d.pfx[jn1]);
        }
        for (int k0 = lane; k0 < cnt; k0 += 2 * LPA) {
            const int k1 = k0 + LPA;
            const bool v1 = k1 < cnt;
            const int j0 = jn0, j1 = jn1;
            const uint4 q0 = qn0, q1 = qn1;
            const int kn = k0 + 2 * LPA;
            if (kn < cnt) {
                jn0 = dbg_index(fx_entry(stage, A, a, kn), d.n, (int)ia, d.status);
                jn1 = kn + LPA < cnt ? dbg_index(fx_entry(stage, A, a, kn + LPA), d.n, (int)ia, d.status) : jn0;
                qn0 = __ldg(&d.pfx[jn0]);
                qn1 = __ldg(&d.pfx[jn1]);
            }
            float2 dx = make_float2(fx_diff(qi.x, q0.x), fx_diff(qi.x, q1.x));
            float2 dy = make_float2(fx_diff(qi.y, q0.y), fx_diff(qi.y, q1.y));
            float2 dz = make_float2(fx_diff(qi.z, q0.z), fx_diff(qi.z, q1.z));
            // the same rounding steps as fx_r2 (FFMA2 rounds each lane as FFMA)
            float2 r2 = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __fmul2_rn(dz, dz)));
            const bool lp0 = HAS_LJ && lj_i && (POT != FX_WATER || fx_oxygen(j0));
            const bool lp1 = HAS_LJ && v1 && lj_i && (POT != FX_WATER || fx_oxygen(j1));
            const bool ep0 = HAS_EL, ep1 = HAS_EL && v1;
            bool lj0, lj1, el0, el1b, amb0, amb1;
            fx_classify(r2.x, lp0, ep0, lj_lo, lj_hi, el_lo, el_hi, lj0, el0, amb0);
            fx_classify(r2.y, lp1, ep1, lj_lo, lj_hi, el_lo, el_hi, lj1, el1b, amb1);
            if (amb0 | amb1) {
                if (amb0) {
                    const FxPair o = fx_pair_fallback(d, s.x, ia, j0, lp0, ep0);
                    lj0 = o.lj_in;
                    el0 = o.el_in;
                    dx.x = o.dx, dy.x = o.dy, dz.x = o.dz, r2.x = o.r2;
                    range_err |= o.range_err != 0;
                }
                if (amb1) {
                    const FxPair o = fx_pair_fallback(d, s.x, ia, j1, lp1, ep1);
                    lj1 = o.lj_in;
                    el1b = o.el_in;
                    dx.y = o.dx, dy.y = o.dy, dz.y = o.dz, r2.y = o.r2;
                    range_err |= o.range_err != 0;
                }
            }
            // pairs outside both cutoffs (and the masked second entry) add
            // nothing; their r^2 is replaced so that no infinity enters
            const bool in0 = lj0 || el0, in1 = lj1 || el1b;
            r2 = make_float2(in0 ? r2.x : 1.0f, in1 ? r2.y : 1.0f);
            float2 f = make_float2(0.f, 0.f);
            if (HAS_LJ) {
                const float2 ri = make_float2(__fdividef(1.0f, r2.x), __fdividef(1.0f, r2.y));
                // s^2 = sigma^2 / r^2 with sigma^2 / u^2 as hi + lo
                const float2 s2 = __ffma2_rn(make_float2(sig2h, sig2h), ri, __fmul2_rn(make_float2(sig2l, sig2l), ri));
                const float2 s6 = __fmul2_rn(__fmul2_rn(s2, s2), s2);
                // (2 s^12 - s^6) / r^2 = (2 s^6 - 1) s^6 / r^2
                const float2 fl = __fmul2_rn(__fmul2_rn(__ffma2_rn(make_float2(2.f, 2.f), s6, make_float2(-1.f, -1.f)), s6),
                                             ri);
                f = make_float2(lj0 ? fl.x : 0.f, lj1 ? fl.y : 0.f);
            }
            if (HAS_EL) {
                const float qj0 = __int_as_float((int)q0.w), qj1 = __int_as_float((int)q1.w);
                const float2 rb = make_float2(rsqrtf(r2.x), rsqrtf(r2.y));
                const float2 r3 = __fmul2_rn(__fmul2_rn(rb, rb), rb);
                const float2 fe = __fmul2_rn(make_float2(kqi * qj0, kqi * qj1), __fadd2_rn(r3, make_float2(-krf, -krf)));
                f = make_float2(el0 ? f.x + fe.x : f.x, el1b ? f.y + fe.y : f.y);
            }
            px = __ffma2_rn(f, dx, px);
            py = __ffma2_rn(f, dy, py);
            pz = __ffma2_rn(f, dz, pz);
        }
        // forces: the two halves, then the lanes
        float hx = __fadd_rn(px.x, px.y), hy = __fadd_rn(py.x, py.y), hz = __fadd_rn(pz.x, pz.y);
        float ex = 0.f, ey = 0.f, ez = 0.f;
#pragma unroll
        for (int o = LPA / 2; o > 0; o >>= 1) {
            fx_join(hx, ex, o, LPA);
            fx_join(hy, ey, o, LPA);
            fx_join(hz, ez, o, LPA);
        }
        if (active && lane == 0) {
            const double im = d.inv_mass[i] * R.fx_fscale;
            const double a0 = ((double)hx + (double)ex) * im, a1 = ((double)hy + (double)ey) * im,
                         a2 = ((double)hz + (double)ez) * im;
            if (!finite64(a0) || !finite64(a1) || !finite64(a2)) status_set(d.status, ST_NONFINITE);
            s.a_new[3 * i] = a0;
            s.a_new[3 * i + 1] = a1;
            s.a_new[3 * i + 2] = a2;
        }
        __syncthreads();  // the stage is read; the next-but-one tile may overwrite it
    }
    if (range_err) status_set(d.status, ST_RANGE);
    if (timeout) {
        if (tid == 0) status_set(d.status, ST_TIMEOUT);
        // the copies this block issued target only its own shared memory;
        // wait (bounded) until they land before the block exits
        for (int st = 0; st < 2; ++st) {
            const int pp = st == 0 ? pend0 : pend1;
            if (pp < 0) continue;
            unsigned tries = 0;
            const unsigned mb = fx_smem(&mbar[st]);
            while (!fx_mbar_try(mb, (unsigned)pp) && ++tries < FX_WAIT_TRIES) {
            }
        }
    }
}

// The same pair arithmetic with the staging per warp: a warp owns tiles of
// AW = 32 / LPA atoms in turn and streams their list rows as 32-entry boxes
// (AW rows x 128 B) through a ring of FXW_SLOTS shared-memory slots, each
// with its own mbarrier; lane 0 keeps up to FXW_SLOTS boxes in flight ahead
// of the lanes, across tile ends. No block barrier: the warps of a block
// run independently, and a tile costs the boxes of its own largest list.
#define FXW_WARPS 8
#define FXW_SLOTS 4

// entry c (< 32) of row a of one swizzled box
__device__ __forceinline__ int fxw_entry(const unsigned char* box, int a, int c)
{
    return *reinterpret_cast<const int*>(box + a * 128 + ((((c >> 2) ^ (a & 7))) << 4) + ((c & 3) << 2));
}

// (LJ alone at 4 lanes per atom, the short rows of the ensembles: 4 CTAs
// per SM at 64 registers beat 3 at 80; the long water rows run faster at 3)
template <int LPA, int POT>
__global__ void __launch_bounds__(FXW_WARPS * 32, (LPA <= 4 && POT == FX_LJ) ? 4 : 3) k_force_fxw(Dev d, StateView s,
                                                                 const __grid_constant__ CUtensorMap map)
{
    static_assert(LPA >= 4 && LPA <= 16, "two entries per lane per box step");
    constexpr int AW = 32 / LPA;    // atoms per warp tile (rows of a box)
    constexpr int IT = 16 / LPA;    // packed steps per box (32 entries / (2 LPA))
    constexpr bool HAS_LJ = POT == FX_LJ || POT == FX_LJEL || POT == FX_WATER;
    constexpr bool HAS_EL = POT == FX_EL || POT == FX_LJEL || POT == FX_WATER;
    __shared__ __align__(8) unsigned long long mbar[FXW_WARPS][FXW_SLOTS];
    extern __shared__ unsigned char fxw_dyn[];
    const int warp = threadIdx.x >> 5, lane_w = threadIdx.x & 31;
    const int lane = lane_w % LPA, a = lane_w / LPA;
    const unsigned dyn = fx_smem(fxw_dyn);
    const unsigned base = ((dyn + 1023u) & ~1023u) + (unsigned)warp * FXW_SLOTS * 1024u;  // slot k: base + 1024 k
    const unsigned char* const slot0 = fxw_dyn + (base - dyn);
    const int64_t ntiles = (d.n + AW - 1) / AW;
    const int64_t nwarps = (int64_t)gridDim.x * FXW_WARPS;
    const int64_t gw = (int64_t)blockIdx.x * FXW_WARPS + warp;
    if (lane_w < FXW_SLOTS) fx_mbar_init(fx_smem(&mbar[warp][lane_w]), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    __syncwarp();

    // a tile's largest list count (warp-uniform)
    auto cmax_of = [&](int64_t t) -> int {
        int c = 0;
        if (lane_w < AW) {
            const int64_t i = t * AW + lane_w;
            if (i < d.n) c = min(d.nbr_count[i], d.nbr_cap);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) c = max(c, __shfl_xor_sync(0xffffffffu, c, o));
        return c;
    };
    // the producer's next box: box pb of the pnb boxes of tile pt
    int64_t pt = gw;
    int pb = 0, pnb = 0;
    while (pt < ntiles && (pnb = (cmax_of(pt) + 31) >> 5) == 0) pt += nwarps;
    unsigned issued = 0, consumed = 0;
    auto refill = [&]() {
        while (pt < ntiles && issued - consumed < FXW_SLOTS) {
            if (lane_w == 0) {
                const unsigned sl = issued % FXW_SLOTS;
                const unsigned mb = fx_smem(&mbar[warp][sl]);
                // the slot was last read by generic loads (ordered by __syncwarp)
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                fx_mbar_expect(mb, AW * 128u);
                fx_tma_box(base + sl * 1024u, &map, pb * 32, (int)(pt * AW), mb);
            }
            ++issued;
            if (++pb >= pnb) {
                pb = 0;
                pt += nwarps;
                while (pt < ntiles && (pnb = (cmax_of(pt) + 31) >> 5) == 0) pt += nwarps;
            }
        }
    };
    refill();

    bool range_err = false, timeout = false;
    for (int64_t t = gw; t < ntiles; t += nwarps) {
        const int cm = cmax_of(t);
        const int nb = (cm + 31) >> 5;
        const int64_t i = t * AW + a;
        const bool active = i < d.n;
        const int64_t ia = active ? i : 0;
        const RepDev& R = d.reps[d.rep_of[ia]];
        const uint4 qi = d.pfx[ia];
        const int cnt = active ? min(d.nbr_count[ia], d.nbr_cap) : 0;
        const bool lj_i = HAS_LJ && (POT != FX_WATER || (ia % 3) == 0);
        const float kqi =
            HAS_EL ? (float)(d.charge[ia] * R.fx_kq) : 0.0f;
        const float lj_lo = R.fx_lj_lo, lj_hi = R.fx_lj_hi, el_lo = R.fx_el_lo, el_hi = R.fx_el_hi;
        const float sig2h = R.fx_sig2_hi, sig2l = R.fx_sig2_lo, krf = R.fx_krf;
        float2 px = make_float2(0.f, 0.f), py = px, pz = px;
        for (int b = 0; b < nb; ++b) {
            const unsigned sl = consumed % FXW_SLOTS;
            const unsigned mb = fx_smem(&mbar[warp][sl]);
            const unsigned parity = (consumed / FXW_SLOTS) & 1u;
            unsigned tries = 0;
            bool late = false;
            while (!fx_mbar_try(mb, parity)) {
                if (++tries > FX_WAIT_TRIES) {
                    late = true;
                    break;
                }
            }
            if (__any_sync(0xffffffffu, late)) {
                timeout = true;
                break;
            }
            const unsigned char* box = slot0 + sl * 1024u;
            const int kb = 32 * b;
            // this box's entries of the lane: kb + lane + 2 m LPA (+ LPA), the
            // next step's entries and gathers issued before this step's
            // arithmetic. No branch per lane: an entry past the row's count
            // gathers the atom itself and adds zero; steps past the tile's
            // largest count are skipped (warp-uniform).
            int jn0, jn1;
            uint4 qn0, qn1;
            {
                const int e0 = fxw_entry(box, a, lane), e1 = fxw_entry(box, a, lane + LPA);
                jn0 = kb + lane < cnt ? dbg_index(e0, d.n, (int)ia, d.status) : (int)ia;
                jn1 = kb + lane + LPA < cnt ? dbg_index(e1, d.n, (int)ia, d.status) : jn0;
                qn0 = __ldg(&d.pfx[jn0]);
                qn1 = __ldg(&d.pfx[jn1]);
            }
#pragma unroll
            for (int m = 0; m < IT; ++m) {
                if (kb + 2 * m * LPA >= cm) break;
                const int c0 = lane + 2 * m * LPA;
                const bool v0 = kb + c0 < cnt, v1 = kb + c0 + LPA < cnt;
                const int j0 = jn0, j1 = jn1;
                const uint4 q0 = qn0, q1 = qn1;
                if (m + 1 < IT && kb + 2 * (m + 1) * LPA < cm) {
                    const int cn = c0 + 2 * LPA;
                    const int e0 = fxw_entry(box, a, cn), e1 = fxw_entry(box, a, cn + LPA);
                    jn0 = kb + cn < cnt ? dbg_index(e0, d.n, (int)ia, d.status) : (int)ia;
                    jn1 = kb + cn + LPA < cnt ? dbg_index(e1, d.n, (int)ia, d.status) : jn0;
                    qn0 = __ldg(&d.pfx[jn0]);
                    qn1 = __ldg(&d.pfx[jn1]);
                }
                fx_pair2<POT>(d, s.x, ia, lj_i, kqi, qi, j0, j1, v0, v1, q0, q1, lj_lo, lj_hi, el_lo, el_hi, sig2h,
                              sig2l, krf, px, py, pz, range_err);
            }
            __syncwarp();  // every lane is done with the slot
            ++consumed;
            refill();
        }
        if (timeout) break;
        float hx = __fadd_rn(px.x, px.y), hy = __fadd_rn(py.x, py.y), hz = __fadd_rn(pz.x, pz.y);
        float ex = 0.f, ey = 0.f, ez = 0.f;
#pragma unroll
        for (int o = LPA / 2; o > 0; o >>= 1) {
            fx_join(hx, ex, o, LPA);
            fx_join(hy, ey, o, LPA);
            fx_join(hz, ez, o, LPA);
        }
        if (active && lane == 0) {
            const double im = d.inv_mass[i] * R.fx_fscale;
            const double a0 = ((double)hx + (double)ex) * im, a1 = ((double)hy + (double)ey) * im,
                         a2 = ((double)hz + (double)ez) * im;
            if (!finite64(a0) || !finite64(a1) || !finite64(a2)) status_set(d.status, ST_NONFINITE);
            s.a_new[3 * i] = a0;
            s.a_new[3 * i + 1] = a1;
            s.a_new[3 * i + 2] = a2;
        }
    }
    if (range_err) status_set(d.status, ST_RANGE);
    if (timeout) {
        if (lane_w == 0) status_set(d.status, ST_TIMEOUT);
        // boxes still in flight land in this warp's own slots: wait (bounded)
        for (unsigned q = consumed; q != issued; ++q) {
            const unsigned mb = fx_smem(&mbar[warp][q % FXW_SLOTS]);
            unsigned tries = 0;
            while (!fx_mbar_try(mb, (q / FXW_SLOTS) & 1u) && ++tries < FX_WAIT_TRIES) {
            }
        }
    }
}

// ---------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------
static PFN_cuTensorMapEncodeTiled_v12000 fx_encode_fn()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    }
    return fn;
}

// The per-warp form runs for 4, 8 and 16 lanes per atom (NBG_FX_BLOCK keeps
// the per-block form, for comparisons), the per-block form for 32.
static bool fx_warp_form(const nbg_ctx* c) { return c->list_lpa <= 16 && !c->fx_block_only; }

// rows (atoms) of one list box of the tensor map
static int fx_box_rows(const nbg_ctx* c) { return fx_warp_form(c) ? 32 / c->list_lpa : FX_THREADS / c->list_lpa; }

// Tensor map of the row-major list: dims (cap entries, n atoms), boxes of
// 32 entries x A atoms, 128-byte swizzle; encoded again whenever the list
// buffer or the lanes per atom change.
int fx_encode_map(nbg_ctx* c)
{
    auto fn = fx_encode_fn();
    if (!fn) {
        c->err = "cuTensorMapEncodeTiled is not available from the driver";
        return NBG_ERR_CUDA;
    }
    CUtensorMap* map = reinterpret_cast<CUtensorMap*>(c->fx_map);
    const cuuint64_t dims[2] = {(cuuint64_t)c->d.nbr_cap, (cuuint64_t)c->n};
    const cuuint64_t strides[1] = {(cuuint64_t)c->d.nbr_cap * sizeof(int)};
    const cuuint32_t box[2] = {32u, (cuuint32_t)fx_box_rows(c)};
    const cuuint32_t estr[2] = {1u, 1u};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_INT32, 2, c->d.nbr, dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        c->err = "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")";
        return NBG_ERR_CUDA;
    }
    return NBG_OK;
}

// Shared memory, opt-in and resident grid of one kernel form: set up once per
// (form, list capacity), outside any stream capture.
template <int LPA, int POT>
static int fx_prepare_form(nbg_ctx* c)
{
    if constexpr (LPA <= 16) {
        if (fx_warp_form(c)) {
            const size_t smem = (size_t)FXW_WARPS * FXW_SLOTS * 1024 + 1024;
            auto kern = k_force_fxw<LPA, POT>;
            if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
                cudaGetLastError();
                return NBG_ERR_UNSUPPORTED;
            }
            int occ = 0;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, FXW_WARPS * 32, smem);
            if (occ < 1) return NBG_ERR_UNSUPPORTED;
            const int64_t ntiles = (c->n + (32 / LPA) - 1) / (32 / LPA);
            c->fx_grid = (int)std::min<int64_t>((ntiles + FXW_WARPS - 1) / FXW_WARPS, (int64_t)c->sms * occ);
            c->fx_smem = smem;
            c->fx_nbox = 0;
            return NBG_OK;
        }
    }
    const int nbox_cap = (c->d.nbr_cap + 31) / 32;
    const size_t smem = 2 * (size_t)nbox_cap * (FX_THREADS / LPA) * 128 + 1024;
    auto kern = k_force_fx<LPA, POT>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return NBG_ERR_UNSUPPORTED;  // the list rows are too long for shared memory
    }
    int occ = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, FX_THREADS, smem);
    if (occ < 1) return NBG_ERR_UNSUPPORTED;
    const int64_t ntiles = (c->n + (FX_THREADS / LPA) - 1) / (FX_THREADS / LPA);
    c->fx_grid = (int)std::min<int64_t>(ntiles, (int64_t)c->sms * occ);
    c->fx_smem = smem;
    c->fx_nbox = nbox_cap;
    return NBG_OK;
}

template <int LPA, int POT>
static void fx_launch(nbg_ctx* c, const StateView& s)
{
    const CUtensorMap* map = reinterpret_cast<const CUtensorMap*>(c->fx_map);
    if constexpr (LPA <= 16) {
        if (fx_warp_form(c)) {
            k_force_fxw<LPA, POT><<<(unsigned)c->fx_grid, FXW_WARPS * 32, c->fx_smem, c->stream>>>(c->d, s, *map);
            return;
        }
    }
    k_force_fx<LPA, POT><<<(unsigned)c->fx_grid, FX_THREADS, c->fx_smem, c->stream>>>(c->d, s, *map, c->fx_nbox);
}

static int fx_pot(const nbg_ctx* c)
{
    if (c->d.kind == NBG_SYSTEM_WATER) return FX_WATER;
    if (c->d.pots == NBG_POT_LJ) return FX_LJ;
    if (c->d.pots == NBG_POT_EL) return FX_EL;
    return FX_LJEL;
}

template <int POT>
static int fx_dispatch(nbg_ctx* c, const StateView* s)
{
    switch (c->list_lpa) {
    case 4: return s ? (fx_launch<4, POT>(c, *s), NBG_OK) : fx_prepare_form<4, POT>(c);
    case 8: return s ? (fx_launch<8, POT>(c, *s), NBG_OK) : fx_prepare_form<8, POT>(c);
    case 16: return s ? (fx_launch<16, POT>(c, *s), NBG_OK) : fx_prepare_form<16, POT>(c);
    case 32: return s ? (fx_launch<32, POT>(c, *s), NBG_OK) : fx_prepare_form<32, POT>(c);
    default: return NBG_ERR_UNSUPPORTED;
    }
}

static int fx_dispatch_pot(nbg_ctx* c, const StateView* s)
{
    switch (fx_pot(c)) {
    case FX_WATER: return fx_dispatch<FX_WATER>(c, s);
    case FX_LJ: return fx_dispatch<FX_LJ>(c, s);
    case FX_EL: return fx_dispatch<FX_EL>(c, s);
    default: return fx_dispatch<FX_LJEL>(c, s);
    }
}

// Make the fixed-point kernel ready for the context's current lanes per atom
// and list capacity (tensor map, shared memory, grid); fx_ready records
// whether it runs (else the split-form kernels do). Called outside capture
// whenever the list buffer or the lanes per atom change.
int fx_prepare(nbg_ctx* c)
{
    c->fx_ready = false;
    if (!c->d.pfx || c->list_lpa < 4 || c->fx_disabled) return NBG_OK;
    int st;
    if ((st = fx_encode_map(c))) return st;
    if (fx_dispatch_pot(c, nullptr) != NBG_OK) return NBG_OK;  // does not fit: split form
    c->fx_ready = true;
    return NBG_OK;
}

// The fixed-point, list-staged force kernel (fx_prepare made it ready).
int launch_force_fx(nbg_ctx* c, const StateView& s)
{
    prof_begin(c);
    fx_dispatch_pot(c, &s);
    prof_end(c);
    NBG_LAUNCH_CHECK(c, "k_force_fx");
    return NBG_OK;
}
