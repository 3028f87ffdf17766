// k_rdf.cu - the radial distribution function's pair histogram
// (rdf, nbody_simulation_result.jl:664-709) over a trajectory of frames.
//
// The reference visits every unordered pair of the LJ participants in every
// saved frame, takes the minimum-image distance under cubic boundaries
// (get_interparticle_distance, boundary_conditions.jl:138-165), and adds 2 to
// bin ceil(r / dr), dr = L / maxbin, when r^2 < (L/2)^2 and 1 < bin <= maxbin.
// The counts are integers, so parity is bit-exact:
//
//   k_rdf_pack    one thread per (frame, participant): wraps the position
//                 into the box, scales it to box units u in [0, 1) and keeps
//                 FP32 u (plain positions, up to RDF_PLAIN_MAXBIN bins) or
//                 splits u into an FP32 hi part on the grid 2^-22 and an FP32
//                 lo remainder (split positions); the image shift of a
//                 difference, rint of it, is exact either way. It also keeps
//                 the unwrapped FP64 position contiguous per frame;
//   k_rdf_pairs   a grid-stride loop over (frame, tile pair) items of
//                 TILE x TILE participants, one i per thread, the j tile in
//                 shared memory as structure-of-arrays float4 groups, two j
//                 per packed FP32x2 instruction. q = r / dr is good to
//                 1.55e-7 maxbin plus ~6 ulp (plain) or ~6 ulp (split). A
//                 pair is undecided when q lies within RDF_MARGIN * q (plus
//                 RDF_MARGIN_ABS * maxbin for plain positions) of an
//                 integer, or r^2 within RDF_MARGIN (plain: twice that) of
//                 (L/2)^2: a bit in a per-thread mask over 32 j, queued in
//                 shared memory once per 32 j, and decided during the next
//                 item by the block with the reference's FP64 arithmetic on
//                 the unwrapped positions (the loop minimum image, r^2, then
//                 bin > b <=> r^2 >= thresh[b], a table the host builds with
//                 IEEE sqrt and division: the reference's ceil(sqrt(r^2) /
//                 dr) exactly). All other pairs go to a per-block shared
//                 histogram by a branch-free add: weight 2 for an
//                 off-diagonal tile pair (each unordered pair once), weight
//                 1 on a diagonal tile, which runs the full square (each
//                 unordered pair twice; a self pair has r = 0, bin 0). A
//                 participant with a coordinate beyond RDF_FAR_BOXES boxes
//                 has a NaN hi part, so all its pairs take the FP64 path:
//                 there the rounding of the reference's long wrap loops can
//                 exceed the band;
//   k_rdf_finish  hist[b] = counts[b].
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "nbg_internal.cuh"

#define RDF_CHUNK 32  // j per undecided-pair mask
#define RDF_QCAP 1024
#define RDF_MAXBIN 16384
// half-width of the band around a bin edge (relative to q) and around
// (L/2)^2 (relative to r^2) in which the FP32 estimate is not trusted; its
// error is below 6 ulp = 3.6e-7
#define RDF_MARGIN 2e-6f
// Plain FP32 box-unit positions (no lo part) for maxbin up to this: each
// component is then off by at most 3 * 2^-25 box (two roundings of u and one
// of the difference; the image shift is exact), |dr| <= sqrt(3) 3 2^-25 L =
// 1.55e-7 L, so q is off by <= 1.55e-7 maxbin, and the band gets
// RDF_MARGIN_ABS * maxbin more (2.6 times that); the half-box band doubles.
#define RDF_PLAIN_MAXBIN 2048
#define RDF_MARGIN_ABS 4e-7
// |coordinate| / L from which a participant's pairs are all decided in FP64.
// Below it the reference's rounding (the difference and up to 2 * 64 wrap
// steps, each within half an ulp of 128 L) stays under 3e-12 L, far inside the
// band (2e-6 dr >= 1.2e-10 L for maxbin <= RDF_MAXBIN).
#define RDF_FAR_BOXES 64.0
// blocks flush their int32 counts after this many items (<= 2^17 counts each)
#define RDF_FLUSH_ITEMS 8192
// q^2 offset of a padding j (beyond any q^2 band)
#define RDF_PAD 1e30f
// host frames go up in at most this many chunks of at least RDF_CHUNK_BYTES,
// each one's kernels starting when it has arrived
#define RDF_MAX_CHUNKS 16
#define RDF_CHUNK_BYTES (8u << 20)

struct RdfArgs {
    const float4* hi;        // [nframes][npad] wrapped hi parts (x, y, z, 0)
    const float4* lo;        // [nframes][npad] lo remainders
    const double4_32a* raw;  // [nframes][npad] the unwrapped positions (x, y, z, 0)
    const double* thresh;    // [maxbin + 1]: bin > b <=> r^2 >= thresh[b]
    int64_t nidx, npad;
    int64_t f0;  // first frame of this launch
    int64_t tiles, tile_pairs, items;
    double L, radius, half2;  // FP64 constants of the reference's formula
    float inv_dr;             // maxbin / L
    float q2scale;            // maxbin^2: (r / dr)^2 from r^2 in box units
    float hq2_lo, hq2_hi;     // (maxbin / 2)^2 band for the half-box test
    float half_thr;           // 1/2 - the absolute part of the bin-edge band
    int maxbin;
    unsigned long long* counts;  // [maxbin] the reference's hist
    unsigned* status;
};

struct RdfPackArgs {
    const double* frames;
    const int32_t* idx;
    float4* hi;
    float4* lo;
    double4_32a* raw;
    int64_t ncols, nidx, npad;
    int64_t f0, nframes;  // the frames of this launch
    double L, invL, far, limit;
    int split;  // hi on the 2^-22 grid and a lo remainder; else plain FP32 u
    unsigned* status;
};

__global__ void __launch_bounds__(256) k_rdf_pack(RdfPackArgs a)
{
    const int64_t tl = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (tl >= a.nframes * a.npad) return;
    const int64_t fl = tl / a.npad, s = tl - fl * a.npad;
    const int64_t f = a.f0 + fl, t = f * a.npad + s;
    float h[3] = {0.f, 0.f, 0.f}, l[3] = {0.f, 0.f, 0.f};
    double4_32a r = make_double4_32a(0.0, 0.0, 0.0, 0.0);
    if (s < a.nidx) {
        const double* p = a.frames + (f * a.ncols + a.idx[s]) * 3;
        r = make_double4_32a(p[0], p[1], p[2], 0.0);
        unsigned st = 0u;
        bool far = false;
        for (int k = 0; k < 3; ++k) {
            const double x = p[k];
            if (!isfinite(x)) {
                st |= ST_NONFINITE;
                continue;
            }
            // coordinates beyond `limit` would take the reference's
            // minimum-image loops more than MINIMAGE_MAX_ITERS passes
            if (fabs(x) > a.limit) {
                st |= ST_RANGE;
                continue;
            }
            far = far || fabs(x) >= a.far;
            double w = fma(-a.L, floor(x * a.invL), x);
            if (w < 0.0) w += a.L;
            if (w >= a.L) w -= a.L;
            const double u = w * a.invL;  // box units, [0, 1]
            if (a.split) {
                const double hq = rint(u * 4194304.0) * (1.0 / 4194304.0);  // the 2^-22 grid
                h[k] = (float)hq;
                l[k] = (float)(u - hq);
            } else {
                h[k] = (float)u;
            }
        }
        if (st) atomicOr(a.status, st);
        if (far || st) h[0] = __int_as_float(0x7fc00000);  // NaN: every pair of this one in FP64
    }
    a.hi[t] = make_float4(h[0], h[1], h[2], 0.f);
    if (a.split) a.lo[t] = make_float4(l[0], l[1], l[2], 0.f);
    a.raw[t] = r;
}

// 1 / sqrt(x) by the approximate hardware instruction, subnormals flushed
// (q^2 below 2^-126 is a self or coincident pair: bin 0 either way)
__device__ __forceinline__ float rsqrt_ftz(float x)
{
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// The decision on one screened pair, without branches. decided: q^2 <= lo
// (inside half the box) and |E| < T (clear of a bin edge: E = q - 1/2 -
// floor(q), T = 1/2 - the margin; NaN, a self pair, counts as clear). A
// decided pair with q > 1 adds w to the shared counter at `slot`, that of
// bin ceil(q). An undecided pair with q^2 < hi, or NaN (a far participant),
// sets `bit` in amb. SELA: the add always runs, at `dummy` (a
// counter of this lane that is never read) for a pair not counted; otherwise
// it is predicated.
template <bool SELA>
__device__ __forceinline__ void rdf_decide(float Q2, float Q, float D, float M, float lo, float hi, unsigned slot,
                                           unsigned dummy, unsigned w, unsigned bit, unsigned& amb)
{
    if (SELA)
        asm volatile(
            "{\n\t"
            ".reg .pred pd, pc, pa;\n\t"
            ".reg .f32 ad;\n\t"
            ".reg .u32 sa;\n\t"
            "abs.f32 ad, %3;\n\t"
            "setp.ltu.f32 pd, ad, %4;\n\t"
            "setp.le.and.f32 pd, %1, %5, pd;\n\t"
            "setp.gt.and.f32 pc, %2, 0f3F800000, pd;\n\t"
            "setp.ltu.and.f32 pa, %1, %6, !pd;\n\t"
            "selp.u32 sa, %7, %8, pc;\n\t"
            "red.shared.add.u32 [sa], %9;\n\t"
            "@pa or.b32 %0, %0, %10;\n\t"
            "}"
            : "+r"(amb)
            : "f"(Q2), "f"(Q), "f"(D), "f"(M), "f"(lo), "f"(hi), "r"(slot), "r"(dummy), "r"(w), "r"(bit));
    else
        asm volatile(
            "{\n\t"
            ".reg .pred pd, pc, pa;\n\t"
            ".reg .f32 ad;\n\t"
            "abs.f32 ad, %3;\n\t"
            "setp.ltu.f32 pd, ad, %4;\n\t"
            "setp.le.and.f32 pd, %1, %5, pd;\n\t"
            "setp.gt.and.f32 pc, %2, 0f3F800000, pd;\n\t"
            "setp.ltu.and.f32 pa, %1, %6, !pd;\n\t"
            "@pc red.shared.add.u32 [%7], %9;\n\t"
            "@pa or.b32 %0, %0, %10;\n\t"
            "}"
            : "+r"(amb)
            : "f"(Q2), "f"(Q), "f"(D), "f"(M), "f"(lo), "f"(hi), "r"(slot), "r"(dummy), "r"(w), "r"(bit));
}

// The reference's arithmetic for one ordered pair: FP64 difference of the
// unwrapped positions, the minimum-image loops, r2 = (x^2 + y^2) + z^2, then
// bin = ceil(sqrt(r2) / dr) as the place of r2 among the thresholds.
// Returns the 1-based bin to count, or 0.
__device__ __forceinline__ int rdf_bin64(const RdfArgs& a, int64_t f, int64_t i, int64_t j)
{
    const double4_32a pi = a.raw[f * a.npad + i], pj = a.raw[f * a.npad + j];
    double x = __dsub_rn(pi.x, pj.x);
    double y = __dsub_rn(pi.y, pj.y);
    double z = __dsub_rn(pi.z, pj.z);
    if (!(wrap_cubic64(x, a.L, a.radius) && wrap_cubic64(y, a.L, a.radius) && wrap_cubic64(z, a.L, a.radius))) {
        atomicOr(a.status, ST_RANGE);
        return 0;
    }
    const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z));
    if (!(r2 < a.half2)) return 0;
    int b = (int)ceilf(sqrtf((float)r2) * a.inv_dr);  // an estimate; the thresholds decide
    b = min(max(b, 1), a.maxbin);
    const double t0 = a.thresh[b - 1], t1 = a.thresh[b];
    if (!(r2 >= t0 && r2 < t1)) {                       // the estimate was off by a bin or more
        while (b > 0 && r2 < a.thresh[b - 1]) --b;      // now bin >= b
        while (b <= a.maxbin && r2 >= a.thresh[b]) ++b; // now bin <= b
    }
    return (b > 1 && b <= a.maxbin) ? b : 0;
}

// TILE participants per tile (threads per block), UNROLL groups of 4 j in
// flight, MINB blocks per SM for the register budget, SELA the form of the
// counting add (rdf_decide), SPLIT hi/lo positions (else plain FP32). The undecided pairs of
// an item are decided during the next item's pair loop (two queues in turn),
// so their FP64 loads overlap the other warps' screening; the next item's
// positions are loaded into registers during the current one.
template <int TILE, int UNROLL, int MINB, bool SELA, bool SPLIT>
__global__ void __launch_bounds__(TILE, MINB) k_rdf_pairs(RdfArgs a)
{
    extern __shared__ unsigned rdf_hist[];  // [maxbin]
    // the j tile: hi x, y, z, (lo x, y, z,) q^2 offset (0, or RDF_PAD past nidx)
    constexpr int NA = SPLIT ? 7 : 4;
    __shared__ __align__(16) float sj[NA][TILE];
    __shared__ unsigned queue[2][RDF_QCAP];  // (i in tile) << 16 | (j in tile)
    __shared__ int qn[2];
    __shared__ long long qf[2], qib[2], qjb[2];  // a queue's frame and tile bases
    __shared__ unsigned qw[2];                   // and weight
    __shared__ unsigned dummies[32];             // SELA: one never-read counter per lane
    const int t = threadIdx.x;
    for (int b = t; b < a.maxbin; b += TILE) rdf_hist[b] = 0u;
    const float magic = 12582912.0f;  // 1.5 * 2^23: x + magic rounds x to an integer
    // q + (2^23 - 1/2) rounds to 2^23 + floor(q) for q >= 1/2 off the integers:
    // the counter of bin ceil(q) = floor(q) + 1 is at 4 bits(that) + slot0
    const float fl_c = 8388607.5f;
    const unsigned slot0 = (unsigned)__cvta_generic_to_shared(rdf_hist) - 4u * 0x4b000000u;
    const unsigned dummy = (unsigned)__cvta_generic_to_shared(dummies) + 4u * (unsigned)(t & 31);
    const float2 m1 = make_float2(-1.f, -1.f);
    const float2 mg = make_float2(magic, magic), mmg = make_float2(-magic, -magic);
    const float2 fc = make_float2(fl_c, fl_c);
    const float2 c2 = make_float2(a.q2scale, a.q2scale);
    const float2 nmarg = make_float2(-RDF_MARGIN, -RDF_MARGIN);
    const float2 hthr = make_float2(a.half_thr, a.half_thr);
    // item -> (frame, tile pair {ti, tj}), tj = ti + s (mod tiles): every unordered pair once
    auto decode = [&](int64_t item, int64_t& f, int64_t& ti, int64_t& tj, int64_t& s) {
        const int64_t fl = item / a.tile_pairs;
        const int64_t p = item - fl * a.tile_pairs;
        f = a.f0 + fl;
        s = p / a.tiles;
        ti = p - s * a.tiles;
        tj = ti + s;
        if (tj >= a.tiles) tj -= a.tiles;
    };
    float4 nh = make_float4(0.f, 0.f, 0.f, 0.f), nl = nh, ih = nh, il = nh;  // the next item's j and i
    if (blockIdx.x < a.items) {
        int64_t f, ti, tj, s;
        decode(blockIdx.x, f, ti, tj, s);
        nh = a.hi[f * a.npad + tj * TILE + t];
        ih = a.hi[f * a.npad + ti * TILE + t];
        if (SPLIT) {
            nl = a.lo[f * a.npad + tj * TILE + t];
            il = a.lo[f * a.npad + ti * TILE + t];
        }
    }
    int since_flush = 0, k = 0;
    for (int64_t item = blockIdx.x; item < a.items; item += gridDim.x, ++k) {
        int64_t f, ti, tj, s;
        decode(item, f, ti, tj, s);
        const int buf = k & 1;
        const int64_t jb = tj * TILE;
        const unsigned w = (s == 0) ? 1u : 2u;
        __syncthreads();  // the previous tile is consumed, this queue's old entries decided
        sj[0][t] = nh.x;
        sj[1][t] = nh.y;
        sj[2][t] = nh.z;
        if (SPLIT) {
            sj[3][t] = nl.x;
            sj[4][t] = nl.y;
            sj[5][t] = nl.z;
        }
        sj[NA - 1][t] = (jb + t < a.nidx) ? 0.f : RDF_PAD;
        if (t == 0) {
            qn[buf] = 0;
            qf[buf] = f;
            qib[buf] = ti * TILE;
            qjb[buf] = jb;
            qw[buf] = w;
        }
        const float4 hi = ih, li = il;
        __syncthreads();
        if (item + gridDim.x < a.items) {
            int64_t f2, ti2, tj2, s2;
            decode(item + gridDim.x, f2, ti2, tj2, s2);
            nh = a.hi[f2 * a.npad + tj2 * TILE + t];
            ih = a.hi[f2 * a.npad + ti2 * TILE + t];
            if (SPLIT) {
                nl = a.lo[f2 * a.npad + tj2 * TILE + t];
                il = a.lo[f2 * a.npad + ti2 * TILE + t];
            }
        }
        if (k > 0) {
            // the previous item's undecided pairs, in FP64
            const int pb = buf ^ 1;
            const int nq = min(qn[pb], RDF_QCAP);
            for (int e = t; e < nq; e += TILE) {
                const unsigned pr = queue[pb][e];
                const int64_t j = qjb[pb] + (pr & 0xffffu);
                if (j < a.nidx) {
                    const int bin = rdf_bin64(a, qf[pb], qib[pb] + (pr >> 16), j);
                    if (bin) atomicAdd(&rdf_hist[bin - 1], qw[pb]);
                }
            }
        }
        const int64_t i = ti * TILE + t;
        if (i < a.nidx) {
            const float2 hx = make_float2(hi.x, hi.x), hy = make_float2(hi.y, hi.y), hz = make_float2(hi.z, hi.z);
            const float2 lx = make_float2(li.x, li.x), ly = make_float2(li.y, li.y), lz = make_float2(li.z, li.z);
            for (int c = 0; c < TILE; c += RDF_CHUNK) {
                unsigned amb = 0u;
#pragma unroll UNROLL
                for (int g = 0; g < RDF_CHUNK; g += 4) {
                    float4 J[NA];
#pragma unroll
                    for (int m = 0; m < NA; ++m) J[m] = *reinterpret_cast<const float4*>(&sj[m][c + g]);
#pragma unroll
                    for (int half = 0; half < 2; ++half) {
                        float2 v[NA];
#pragma unroll
                        for (int m = 0; m < NA; ++m) v[m] = half ? make_float2(J[m].z, J[m].w) : make_float2(J[m].x, J[m].y);
                        // differences in box units, the image shift s = rint(dh); dh - s is exact
                        const float2 dxh = __ffma2_rn(v[0], m1, hx), dyh = __ffma2_rn(v[1], m1, hy);
                        const float2 dzh = __ffma2_rn(v[2], m1, hz);
                        const float2 sx = __fadd2_rn(__fadd2_rn(dxh, mg), mmg);
                        const float2 sy = __fadd2_rn(__fadd2_rn(dyh, mg), mmg);
                        const float2 sz = __fadd2_rn(__fadd2_rn(dzh, mg), mmg);
                        float2 dx = __ffma2_rn(sx, m1, dxh), dy = __ffma2_rn(sy, m1, dyh), dz = __ffma2_rn(sz, m1, dzh);
                        if (SPLIT) {  // the lo differences
                            dx = __fadd2_rn(dx, __ffma2_rn(v[3], m1, lx));
                            dy = __fadd2_rn(dy, __ffma2_rn(v[4], m1, ly));
                            dz = __fadd2_rn(dz, __ffma2_rn(v[5], m1, lz));
                        }
                        const float2 r2 = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __fmul2_rn(dz, dz)));
                        const float2 q2 = __ffma2_rn(r2, c2, v[NA - 1]);  // (r / dr)^2, or past the band for padding
                        // q = sqrt(q2); q2 = 0 (a self pair) gives NaN: clear, not counted
                        const float2 q = __fmul2_rn(q2, make_float2(rsqrt_ftz(q2.x), rsqrt_ftz(q2.y)));
                        const float2 tq = __fadd2_rn(q, fc);                    // 2^23 + floor(q)
                        const float2 e = __fadd2_rn(q, __ffma2_rn(tq, m1, fc));  // q - 1/2 - floor(q), exact
                        const float2 thr = __ffma2_rn(q, nmarg, hthr);          // 1/2 - the band
                        const unsigned sl0 = slot0 + 4u * __float_as_uint(tq.x);
                        const unsigned sl1 = slot0 + 4u * __float_as_uint(tq.y);
                        const int p0 = g + 2 * half;
                        rdf_decide<SELA>(q2.x, q.x, e.x, thr.x, a.hq2_lo, a.hq2_hi, sl0, dummy, w, 1u << p0, amb);
                        rdf_decide<SELA>(q2.y, q.y, e.y, thr.y, a.hq2_lo, a.hq2_hi, sl1, dummy, w, 2u << p0, amb);
                    }
                }
                if (amb) {  // this chunk's undecided pairs, for the FP64 pass
                    int slot = atomicAdd(&qn[buf], __popc(amb));
                    while (amb) {
                        const int b = __ffs(amb) - 1;
                        amb &= amb - 1u;
                        if (slot < RDF_QCAP) {
                            queue[buf][slot] = ((unsigned)t << 16) | (unsigned)(c + b);
                        } else if (jb + c + b < a.nidx) {
                            const int bin = rdf_bin64(a, f, i, jb + c + b);
                            if (bin) atomicAdd(&rdf_hist[bin - 1], w);
                        }
                        ++slot;
                    }
                }
            }
        }
        if (++since_flush == RDF_FLUSH_ITEMS) {
            // bounded int32 counters: move them to the 64-bit totals (atomically,
            // other threads may still be counting)
            since_flush = 0;
            for (int b = t; b < a.maxbin; b += TILE) {
                const unsigned cnt = atomicExch(&rdf_hist[b], 0u);
                if (cnt) atomicAdd(a.counts + b, (unsigned long long)cnt);
            }
        }
    }
    __syncthreads();
    if (k > 0) {  // the last item's undecided pairs
        const int pb = (k - 1) & 1;
        const int nq = min(qn[pb], RDF_QCAP);
        for (int e = t; e < nq; e += TILE) {
            const unsigned pr = queue[pb][e];
            const int64_t j = qjb[pb] + (pr & 0xffffu);
            if (j < a.nidx) {
                const int bin = rdf_bin64(a, qf[pb], qib[pb] + (pr >> 16), j);
                if (bin) atomicAdd(&rdf_hist[bin - 1], qw[pb]);
            }
        }
    }
    __syncthreads();
    for (int b = t; b < a.maxbin; b += TILE) {
        const unsigned cnt = rdf_hist[b];
        if (cnt) atomicAdd(a.counts + b, (unsigned long long)cnt);
    }
}

__global__ void k_rdf_finish(const unsigned long long* counts, int maxbin, double* hist)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b < maxbin) hist[b] = (double)counts[b];
}

// The instantiated forms of k_rdf_pairs, each with plain positions (maxbin up
// to RDF_PLAIN_MAXBIN) and split ones; NBG_RDF_FORM=<index> picks one
// (default 0: 4.17 ms on the 4096-oxygen, 512-frame water trajectory against
// 4.20-4.92 ms for the others).
struct RdfForm {
    void (*plain)(RdfArgs);
    void (*split)(RdfArgs);
    int tile, unroll, minb;
};
#define RDF_FORM(T, U, M, S) {k_rdf_pairs<T, U, M, S, false>, k_rdf_pairs<T, U, M, S, true>, T, U, M}
const RdfForm kRdfForms[] = {
    RDF_FORM(256, 8, 3, true), RDF_FORM(256, 8, 3, false), RDF_FORM(256, 8, 2, true),
    RDF_FORM(256, 8, 4, true), RDF_FORM(128, 8, 6, true), RDF_FORM(128, 8, 4, false),
};
#undef RDF_FORM
const int kRdfFormCount = (int)(sizeof(kRdfForms) / sizeof(kRdfForms[0]));

namespace {

// Scratch of the histogram, kept across calls on the same device and grown
// on demand; one call at a time.
struct RdfScratch {
    int device = -1;
    double* frames = nullptr;
    size_t frames_cap = 0;
    double4_32a* packed = nullptr;  // N float4 hi, N float4 lo, N double4 raw (2 N double4_32a)
    size_t packed_cap = 0;
    int32_t* idx = nullptr;
    size_t idx_cap = 0;
    std::vector<int32_t> idx_host;  // what idx holds
    unsigned long long* counts = nullptr;
    double* hist = nullptr;
    double* thresh = nullptr;  // [RDF_MAXBIN + 1]
    double thresh_L = 0.0;     // the box and bin count thresh was built for
    int thresh_maxbin = 0;
    unsigned* status = nullptr;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};  // pack start/end, pairs start/end
    cudaStream_t copy = nullptr, comp = nullptr;  // host frames: chunk uploads, and the kernels behind them
    cudaEvent_t copied[RDF_MAX_CHUNKS] = {};      // chunk c is on the device
    double last_ms[2] = {0.0, 0.0};                             // the last call's pack, pairs
    int sms = 0;
    int form = 0;        // index into kRdfForms
    int occ_maxbin = 0;  // the histogram size pair_blocks was sized for
    int pair_blocks = 0;
};

std::mutex g_rdf_mutex;
RdfScratch g_rdf;

void rdf_release(RdfScratch& s)
{
    for (cudaEvent_t& e : s.ev)
        if (e) cudaEventDestroy(e);
    for (cudaEvent_t& e : s.copied)
        if (e) cudaEventDestroy(e);
    if (s.copy) cudaStreamDestroy(s.copy);
    if (s.comp) cudaStreamDestroy(s.comp);
    cudaFree(s.frames);
    cudaFree(s.packed);
    cudaFree(s.idx);
    cudaFree(s.counts);
    cudaFree(s.hist);
    cudaFree(s.thresh);
    cudaFree(s.status);
    s = RdfScratch();
}

template <class T>
bool grow(T*& p, size_t& cap, size_t n)
{
    if (n <= cap) return true;
    cudaFree(p);
    p = nullptr;
    cap = 0;
    if (cudaMalloc(&p, n * sizeof(T)) != cudaSuccess) return false;
    cap = n;
    return true;
}

// The smallest r^2 >= 0 whose bin ceil(sqrt(r^2) / dr) exceeds b, with the
// reference's IEEE double sqrt and division (nbody_simulation_result.jl:683):
// bin > b <=> sqrt(r2) / dr > b, monotone in r2, found by bisection over the
// ordered bit patterns of the non-negative doubles.
double rdf_threshold(double dr, int b)
{
    uint64_t lo = 0, hi = 0x7ff0000000000000ull;  // 0 (false) and +inf (true)
    while (hi - lo > 1) {
        const uint64_t mid = lo + (hi - lo) / 2;
        double x;
        std::memcpy(&x, &mid, sizeof x);
        if (std::sqrt(x) / dr > (double)b)
            hi = mid;
        else
            lo = mid;
    }
    double x;
    std::memcpy(&x, &hi, sizeof x);
    return x;
}

bool is_device_pointer(const void* p)
{
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

}  // namespace

extern "C" int nbg_rdf_histogram(const double* frames, int64_t nframes, int64_t ncols, const int32_t* idx,
                                 int64_t nidx, double L, int32_t maxbin, int device, double* hist)
{
    NBG_RANGE("nbg_rdf_histogram");
    if (!hist || nframes < 0 || ncols < 0 || nidx < 0 || !(L > 0.0) || !std::isfinite(L) || maxbin < 1 ||
        maxbin > RDF_MAXBIN || nidx > (int64_t)1 << 30)
        return NBG_ERR_ARG;
    if (nframes > 0 && nidx > 0 && !frames) return NBG_ERR_ARG;
    if (nidx > 0 && !idx) return NBG_ERR_ARG;
    for (int64_t a = 0; a < nidx; ++a)
        if (idx[a] < 0 || idx[a] >= ncols) return NBG_ERR_ARG;
    std::lock_guard<std::mutex> lock(g_rdf_mutex);
    if (cudaSetDevice(device) != cudaSuccess) return NBG_ERR_CUDA;
    RdfScratch& S = g_rdf;
    if (S.device != device) {
        if (S.device >= 0) {
            int cur = device;
            cudaSetDevice(S.device);
            rdf_release(S);
            cudaSetDevice(cur);
        }
        S.device = device;
        if (cudaMalloc(&S.counts, RDF_MAXBIN * sizeof(unsigned long long)) != cudaSuccess ||
            cudaMalloc(&S.hist, RDF_MAXBIN * sizeof(double)) != cudaSuccess ||
            cudaMalloc(&S.thresh, (RDF_MAXBIN + 1) * sizeof(double)) != cudaSuccess ||
            cudaMalloc(&S.status, sizeof(unsigned)) != cudaSuccess) {
            rdf_release(S);
            return NBG_ERR_NOMEM;
        }
        bool ok = cudaStreamCreateWithFlags(&S.copy, cudaStreamNonBlocking) == cudaSuccess &&
                  cudaStreamCreateWithFlags(&S.comp, cudaStreamNonBlocking) == cudaSuccess;
        for (cudaEvent_t& e : S.ev) ok = ok && cudaEventCreate(&e) == cudaSuccess;
        for (cudaEvent_t& e : S.copied) ok = ok && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess;
        if (!ok) {
            rdf_release(S);
            return NBG_ERR_CUDA;
        }
        cudaDeviceGetAttribute(&S.sms, cudaDevAttrMultiProcessorCount, device);
        for (const RdfForm& fm : kRdfForms) {
            cudaFuncSetAttribute(fm.plain, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 RDF_MAXBIN * (int)sizeof(unsigned));
            cudaFuncSetAttribute(fm.split, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 RDF_MAXBIN * (int)sizeof(unsigned));
        }
        const char* env = std::getenv("NBG_RDF_FORM");
        S.form = env ? std::atoi(env) : 0;
        if (S.form < 0 || S.form >= kRdfFormCount) S.form = 0;
    }
    const RdfForm& form = kRdfForms[S.form];
    const bool split = maxbin > RDF_PLAIN_MAXBIN;
    void (*const pairs_kernel)(RdfArgs) = split ? form.split : form.plain;
    if (S.occ_maxbin != maxbin) {
        // a grid of all the blocks that fit at once with this histogram size
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pairs_kernel, form.tile, maxbin * sizeof(unsigned));
        S.pair_blocks = S.sms * std::max(per_sm, 1);
        S.occ_maxbin = maxbin;
    }
    const bool work = nframes > 0 && nidx > 0;
    // host frames: uploaded in chunks on S.copy, the kernels on S.comp behind
    // them; device frames: the legacy default stream (ordered after the
    // caller's work there)
    const bool host_in = work && !is_device_pointer(frames);
    cudaStream_t st = host_in ? S.comp : 0;
    const bool dev_out = is_device_pointer(hist);
    double* hist_d = dev_out ? hist : S.hist;
    cudaMemsetAsync(S.counts, 0, maxbin * sizeof(unsigned long long), st);
    cudaMemsetAsync(S.status, 0, sizeof(unsigned), st);
    const int64_t tiles = (nidx + form.tile - 1) / form.tile;
    const int64_t npad = tiles * form.tile;
    if (work) {
        const size_t frame_doubles = (size_t)ncols * 3;
        int64_t per_chunk = nframes;
        if (host_in) {
            const double bytes = (double)nframes * frame_doubles * sizeof(double);
            const int64_t want = std::max<int64_t>(1, std::min<int64_t>(RDF_MAX_CHUNKS, (int64_t)(bytes / RDF_CHUNK_BYTES)));
            per_chunk = (nframes + want - 1) / want;
        }
        const int64_t nchunks = (nframes + per_chunk - 1) / per_chunk;
        const size_t nslots = (size_t)nframes * (size_t)npad;
        // every allocation before the first asynchronous copy from the
        // caller's frames, so that no early return leaves one in flight
        if (!grow(S.packed, S.packed_cap, 2 * nslots)) return NBG_ERR_NOMEM;
        if (S.idx_cap < (size_t)nidx) {
            S.idx_host.clear();  // a new buffer: upload the columns again
            if (!grow(S.idx, S.idx_cap, (size_t)nidx)) return NBG_ERR_NOMEM;
        }
        if (host_in && !grow(S.frames, S.frames_cap, (size_t)nframes * frame_doubles)) return NBG_ERR_NOMEM;
        // an error after the uploads started waits for them before returning
        auto bail = [&](int code) {
            if (host_in) cudaStreamSynchronize(S.copy);
            return code;
        };
        const double* frames_d = frames;
        if (host_in) {
            for (int64_t c = 0; c < nchunks; ++c) {
                const int64_t f0 = c * per_chunk, fn = std::min(per_chunk, nframes - f0);
                if (cudaMemcpyAsync(S.frames + f0 * frame_doubles, frames + f0 * frame_doubles,
                                    (size_t)fn * frame_doubles * sizeof(double), cudaMemcpyHostToDevice,
                                    S.copy) != cudaSuccess)
                    return bail(NBG_ERR_CUDA);
                cudaEventRecord(S.copied[c], S.copy);
            }
            frames_d = S.frames;
        }
        if (S.idx_host.size() != (size_t)nidx ||
            std::memcmp(S.idx_host.data(), idx, (size_t)nidx * sizeof(int32_t)) != 0) {
            S.idx_host.assign(idx, idx + nidx);
            if (cudaMemcpyAsync(S.idx, S.idx_host.data(), (size_t)nidx * sizeof(int32_t), cudaMemcpyHostToDevice,
                                st) != cudaSuccess)
                return bail(NBG_ERR_CUDA);
        }
        if (S.thresh_L != L || S.thresh_maxbin != maxbin) {
            const double dr = L / maxbin;  // pbc.L / maxbin
            std::vector<double> th(maxbin + 1);
            for (int b = 0; b <= maxbin; ++b) th[b] = rdf_threshold(dr, b);
            if (cudaMemcpy(S.thresh, th.data(), th.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess)
                return bail(NBG_ERR_CUDA);
            S.thresh_L = L;
            S.thresh_maxbin = maxbin;
        }
        RdfPackArgs pa;
        pa.frames = frames_d;
        pa.idx = S.idx;
        pa.hi = reinterpret_cast<float4*>(S.packed);
        pa.lo = pa.hi + nslots;
        pa.raw = S.packed + nslots;
        pa.ncols = ncols;
        pa.nidx = nidx;
        pa.npad = npad;
        pa.L = L;
        pa.invL = 1.0 / L;
        pa.far = RDF_FAR_BOXES * L;
        pa.split = split ? 1 : 0;
        pa.limit = 0.25 * MINIMAGE_MAX_ITERS * L;
        pa.status = S.status;

        RdfArgs a;
        a.hi = pa.hi;
        a.lo = pa.lo;
        a.raw = pa.raw;
        a.thresh = S.thresh;
        a.nidx = nidx;
        a.npad = npad;
        a.tiles = tiles;
        a.tile_pairs = tiles * (tiles + 1) / 2;
        a.L = L;
        a.radius = 0.5 * L;
        a.inv_dr = (float)(maxbin / L);
        a.half2 = (0.5 * L) * (0.5 * L);
        const double qmax = 0.5 * maxbin;  // q = r / dr at r = L / 2
        a.q2scale = (float)((double)maxbin * maxbin);
        const double hband = split ? RDF_MARGIN : 2.0 * RDF_MARGIN;
        a.hq2_lo = (float)(qmax * qmax * (1.0 - hband));
        a.hq2_hi = (float)(qmax * qmax * (1.0 + hband));
        a.half_thr = (float)(0.5 - (split ? 0.0 : RDF_MARGIN_ABS * maxbin));
        a.maxbin = maxbin;
        a.counts = S.counts;
        a.status = S.status;

        for (int64_t c = 0; c < nchunks; ++c) {
            const int64_t f0 = c * per_chunk, fn = std::min(per_chunk, nframes - f0);
            if (host_in) cudaStreamWaitEvent(st, S.copied[c], 0);
            if (c == 0) cudaEventRecord(S.ev[0], st);
            pa.f0 = f0;
            pa.nframes = fn;
            const int64_t pack_threads = fn * npad;
            k_rdf_pack<<<(unsigned)((pack_threads + 255) / 256), 256, 0, st>>>(pa);
            if (!host_in) {
                // device frames, one chunk: invalid coordinates end the call
                // here (their pairs would all take the FP64 path)
                cudaEventRecord(S.ev[1], st);
                unsigned pst = 0;
                if (cudaMemcpyAsync(&pst, S.status, sizeof(unsigned), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                    cudaStreamSynchronize(st) != cudaSuccess)
                    return NBG_ERR_CUDA;
                if (pst & ST_NONFINITE) return NBG_ERR_NONFINITE;
                if (pst & ST_RANGE) return NBG_ERR_RANGE;
                cudaEventRecord(S.ev[2], st);
            }
            a.f0 = f0;
            a.items = fn * a.tile_pairs;
            const int64_t blocks = std::min<int64_t>(a.items, S.pair_blocks);
            pairs_kernel<<<(unsigned)blocks, form.tile, maxbin * sizeof(unsigned), st>>>(a);
        }
        cudaEventRecord(S.ev[3], st);
    }
    k_rdf_finish<<<(maxbin + 255) / 256, 256, 0, st>>>(S.counts, maxbin, hist_d);
    if (!dev_out &&
        cudaMemcpyAsync(hist, hist_d, maxbin * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess)
        return NBG_ERR_CUDA;
    unsigned status = 0;
    if (cudaMemcpyAsync(&status, S.status, sizeof(unsigned), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return NBG_ERR_CUDA;
    if (cudaGetLastError() != cudaSuccess) return NBG_ERR_CUDA;
    S.last_ms[0] = S.last_ms[1] = 0.0;
    if (work) {
        float ms = 0.f;
        if (host_in) {  // the pipelined chunks as a whole
            if (cudaEventElapsedTime(&ms, S.ev[0], S.ev[3]) == cudaSuccess) S.last_ms[1] = ms;
        } else {
            if (cudaEventElapsedTime(&ms, S.ev[0], S.ev[1]) == cudaSuccess) S.last_ms[0] = ms;
            if (cudaEventElapsedTime(&ms, S.ev[2], S.ev[3]) == cudaSuccess) S.last_ms[1] = ms;
        }
    }
    if (status & ST_NONFINITE) return NBG_ERR_NONFINITE;
    if (status & ST_RANGE) return NBG_ERR_RANGE;
    return NBG_OK;
}

extern "C" int nbg_rdf_kernel_times(double* ms)
{
    if (!ms) return NBG_ERR_ARG;
    std::lock_guard<std::mutex> lock(g_rdf_mutex);
    ms[0] = g_rdf.last_ms[0];
    ms[1] = g_rdf.last_ms[1];
    return NBG_OK;
}
