// k_forces.cu - force kernels.
//
//  k_gravity<PLAIN>  all-pairs gravity (gravitational_acceleration!,
//                    basic_potentials.jl:306-331): 128-body j-tiles of split
//                    positions staged in shared memory and read as warp-wide
//                    broadcasts, two bodies i per thread; the j range is cut
//                    into J chunks so the grid fills whole waves of resident
//                    blocks (J partials per body in scratch, reduced in fixed
//                    order by k_gravity_reduce).
//                    Per pair: FP32 differences of hi/lo split positions (exact
//                    to ~2^-24 of |r_ij|, or plain FP32 positions when PLAIN),
//                    one rsqrt, partial sums per tile folded into a compensated
//                    (TwoSum) pair. With tile boxes (bodies sorted along a
//                    Morton curve), a tile pair whose boxes or radial shells
//                    are apart by at least 1/16 of their largest |r| uses the
//                    plain difference: its error, 2^-24 of the coordinates,
//                    is then below 2^-19 of |r_ij|.
//  k_allpairs        every other potential on small / unbounded systems, all
//                    pairs through shared-memory tiles, same pair code as the
//                    list kernel plus gravity and the magnetic dipole term.
//  k_force_list      cutoff LJ + reaction-field electrostatics over a Verlet
//                    list (one thread per atom, coalesced column-major list).
//  k_bonded          SPC/Fw harmonic bonds and H-O-H angles, one thread per
//                    molecule (basic_potentials.jl:367-433), FP32 terms from
//                    FP64 intramolecular differences.
#include <cub/device/device_radix_sort.cuh>

#include "nbg_internal.cuh"

#define GB 128         // gravity block size = j-tile size
#define GI_MAX (4 * GB)  // bodies i per block at most (TI <= 4)

__device__ __forceinline__ float rsqrt_ftz(float x)
{
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Grid: (i-block, j-chunk) units; each thread owns TI bodies i (strided by
// GB within the block) and walks the chunk's j-tiles from shared memory:
// every lane of a warp reads the same body j (one broadcast load serves TI
// pairs). PACKED evaluates the TI bodies two at a time with the packed
// FP32x2 instructions (__ffma2_rn / __fadd2_rn / __fmul2_rn), which halve the
// issued FP32 instructions; both forms round every element identically.
// Per pair: p += m_j (r_i - r_j) |r_i - r_j|^-3 (gravitational_acceleration!,
// basic_potentials.jl:318-324), the j == i term skipped (:318).
// Accumulate one j-tile (sh_hi / sh_lo) into the per-body partials.
// DIAG: the tile holds some of this thread's own bodies (j == i skipped).
template <bool PLAIN, int TI, bool PACKED, bool DIAG, bool UNIFORM>
__device__ __forceinline__ void grav_tile(const float4* sh_hi, const float4* sh_lo, int64_t j0, const int64_t* ii,
                                          const float* hx, const float* hy, const float* hz, const float* lx,
                                          const float* ly, const float* lz, float* px, float* py, float* pz)
{
    constexpr int NP = PACKED ? TI / 2 : 1;
    if (!PACKED) {
#pragma unroll 4
        for (int jj = 0; jj < GB; ++jj) {
            const float4 hj = sh_hi[jj];
            float4 lj = make_float4(0.f, 0.f, 0.f, 0.f);
            if (!PLAIN) lj = sh_lo[jj];
#pragma unroll
            for (int k = 0; k < TI; ++k) {
                float dx = hx[k] - hj.x, dy = hy[k] - hj.y, dz = hz[k] - hj.z;
                if (!PLAIN) {
                    dx += lx[k] - lj.x;
                    dy += ly[k] - lj.y;
                    dz += lz[k] - lj.z;
                }
                float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                float ri = rsqrt_ftz(r2);
                if (DIAG && j0 + jj == ii[k]) ri = 0.0f;
                float sc = hj.w * ri * (ri * ri);
                px[k] = fmaf(sc, dx, px[k]);
                py[k] = fmaf(sc, dy, py[k]);
                pz[k] = fmaf(sc, dz, pz[k]);
            }
        }
        return;
    }
    float2 hx2[NP], hy2[NP], hz2[NP], lx2[NP], ly2[NP], lz2[NP], px2[NP], py2[NP], pz2[NP];
#pragma unroll
    for (int q = 0; q < NP; ++q) {
        hx2[q] = make_float2(hx[2 * q], hx[2 * q + 1]);
        hy2[q] = make_float2(hy[2 * q], hy[2 * q + 1]);
        hz2[q] = make_float2(hz[2 * q], hz[2 * q + 1]);
        lx2[q] = make_float2(lx[2 * q], lx[2 * q + 1]);
        ly2[q] = make_float2(ly[2 * q], ly[2 * q + 1]);
        lz2[q] = make_float2(lz[2 * q], lz[2 * q + 1]);
        px2[q] = py2[q] = pz2[q] = make_float2(0.f, 0.f);
    }
    const float2 m1 = make_float2(-1.f, -1.f);
#pragma unroll 8
    for (int jj = 0; jj < GB; ++jj) {
        const float4 hj = sh_hi[jj];
        const float2 jx = make_float2(hj.x, hj.x), jy = make_float2(hj.y, hj.y), jz = make_float2(hj.z, hj.z);
        const float2 jm = make_float2(hj.w, hj.w);
        float2 kx = m1, ky = m1, kz = m1;
        if (!PLAIN) {
            const float4 lj = sh_lo[jj];
            kx = make_float2(lj.x, lj.x);
            ky = make_float2(lj.y, lj.y);
            kz = make_float2(lj.z, lj.z);
        }
#pragma unroll
        for (int q = 0; q < NP; ++q) {
            float2 dx = __ffma2_rn(jx, m1, hx2[q]);  // hi_i - hi_j (scaling by -1 is exact)
            float2 dy = __ffma2_rn(jy, m1, hy2[q]);
            float2 dz = __ffma2_rn(jz, m1, hz2[q]);
            if (!PLAIN) {
                dx = __fadd2_rn(dx, __ffma2_rn(kx, m1, lx2[q]));
                dy = __fadd2_rn(dy, __ffma2_rn(ky, m1, ly2[q]));
                dz = __fadd2_rn(dz, __ffma2_rn(kz, m1, lz2[q]));
            }
            float2 r2 = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __fmul2_rn(dz, dz)));
            float2 ri = make_float2(rsqrt_ftz(r2.x), rsqrt_ftz(r2.y));
            if (DIAG) {
                if (j0 + jj == ii[2 * q]) ri.x = 0.0f;
                if (j0 + jj == ii[2 * q + 1]) ri.y = 0.0f;
            }
            // equal masses: m_j leaves the sum (the reduction multiplies by G m)
            float2 sc = UNIFORM ? __fmul2_rn(ri, __fmul2_rn(ri, ri)) : __fmul2_rn(__fmul2_rn(jm, ri), __fmul2_rn(ri, ri));
            px2[q] = __ffma2_rn(sc, dx, px2[q]);
            py2[q] = __ffma2_rn(sc, dy, py2[q]);
            pz2[q] = __ffma2_rn(sc, dz, pz2[q]);
        }
    }
#pragma unroll
    for (int q = 0; q < NP; ++q) {
        px[2 * q] = px2[q].x; px[2 * q + 1] = px2[q].y;
        py[2 * q] = py2[q].x; py[2 * q + 1] = py2[q].y;
        pz[2 * q] = pz2[q].x; pz[2 * q + 1] = pz2[q].y;
    }
}

// Grid: (i-block, j-chunk) units; each thread owns TI bodies i (strided by
// GB within the block) and walks the chunk's j-tiles from shared memory:
// every lane of a warp reads the same body j (one broadcast load serves TI
// pairs). PACKED evaluates the TI bodies two at a time with the packed
// FP32x2 instructions (__ffma2_rn / __fadd2_rn / __fmul2_rn), which halve the
// issued FP32 instructions; both forms round every element identically.
// Per pair: p += m_j (r_i - r_j) |r_i - r_j|^-3 (gravitational_acceleration!,
// basic_potentials.jl:318-324), the j == i term skipped (:318).
// UNIFORM: every body has the same mass, which the reduction applies.
template <bool PLAIN, int TI, bool PACKED, bool UNIFORM>
__global__ void __launch_bounds__(GB, TI == 2 ? 7 : 1) k_gravity(const float4* __restrict__ phi, const float4* __restrict__ plo,
                                                int64_t n, int64_t npad, int jchunks, double* __restrict__ part,
                                                const float4* __restrict__ box, float far2)
{
    static_assert(TI == 1 || TI == 2 || TI == 4, "TI");
    static_assert(!PACKED || TI >= 2, "packed needs pairs");
    static_assert(PACKED || !UNIFORM, "the uniform-mass form is packed");
    __shared__ float4 sh_hi[GB];
    __shared__ float4 sh_lo[PLAIN ? 1 : GB];
    const int64_t ntile = npad / GB;
    const int64_t iblock = blockIdx.x / jchunks;
    const int jc = (int)(blockIdx.x % jchunks);
    const int64_t t0 = (int64_t)jc * ntile / jchunks;
    const int64_t t1 = (int64_t)(jc + 1) * ntile / jchunks;
    const int64_t ib0 = iblock * (TI * GB);
    // thread t owns bodies ib0 + TI t .. + TI - 1: a warp's bodies lie in one
    // of the block's TI 128-body tiles (its i-tile `it`), so the far test of a
    // tile pair is uniform over the warp
    const int it = (int)((threadIdx.x * TI) / GB);
    float hx[TI], hy[TI], hz[TI], lx[TI], ly[TI], lz[TI];
    int64_t ii[TI];
#pragma unroll
    for (int k = 0; k < TI; ++k) {
        ii[k] = ib0 + (int64_t)threadIdx.x * TI + k;
        float4 h = phi[ii[k]];
        hx[k] = h.x; hy[k] = h.y; hz[k] = h.z;
        float4 l = PLAIN ? make_float4(0.f, 0.f, 0.f, 0.f) : plo[ii[k]];
        lx[k] = l.x; ly[k] = l.y; lz[k] = l.z;
    }
    Acc2 ax[TI], ay[TI], az[TI];
#pragma unroll
    for (int k = 0; k < TI; ++k) ax[k] = ay[k] = az[k] = Acc2{0.f, 0.f};
    // boxes and radial shells of the block's TI i-tiles
    __shared__ float4 ibox_s[2 * TI];
    if (!PLAIN && box && threadIdx.x < 2 * TI) ibox_s[threadIdx.x] = box[2 * (ib0 / GB) + threadIdx.x];
    constexpr unsigned ALL_FAR = (1u << TI) - 1u;
    __shared__ unsigned char far_s[GB];  // per j-tile of the next GB: bit k = far from i-tile k
    for (int64_t t = t0; t < t1; ++t) {
        const int64_t j0 = t * GB;
        // far tile pair: a lower bound g of |r_ij| (the boxes' gap, or the
        // radial shells' gap) with F g >= the largest |r| of both tiles
        // (far2 = F^2; F = 16 by default);
        // flags for GB j-tiles at a time, one j-tile per thread
        if (!PLAIN && box && (t - t0) % GB == 0) {
            __syncthreads();
            const int64_t tt = t + threadIdx.x;
            unsigned f = 0;
            if (tt < t1) {
                const float4 lo4 = box[2 * tt], hi4 = box[2 * tt + 1];
#pragma unroll
                for (int k = 0; k < TI; ++k) {
                    const float4 a = ibox_s[2 * k], b = ibox_s[2 * k + 1];  // (min x,y,z, max|r|), (max x,y,z, min|r|)
                    const float gx = fmaxf(0.f, fmaxf(a.x - hi4.x, lo4.x - b.x));
                    const float gy = fmaxf(0.f, fmaxf(a.y - hi4.y, lo4.y - b.y));
                    const float gz = fmaxf(0.f, fmaxf(a.z - hi4.z, lo4.z - b.z));
                    const float gr = fmaxf(0.f, fmaxf(b.w - lo4.w, hi4.w - a.w));
                    const float g2 = fmaxf(gx * gx + gy * gy + gz * gz, gr * gr);
                    const float mm = fmaxf(a.w, lo4.w);
                    if (g2 > 0.f && far2 * g2 >= mm * mm) f |= 1u << k;
                }
            }
            far_s[threadIdx.x] = (unsigned char)f;
        }
        __syncthreads();
        const unsigned fl = (!PLAIN && box) ? far_s[(t - t0) % GB] : 0u;
        const bool far = (fl >> it) & 1u;
        sh_hi[threadIdx.x] = phi[j0 + threadIdx.x];
        if (!PLAIN && fl != ALL_FAR) sh_lo[threadIdx.x] = plo[j0 + threadIdx.x];
        __syncthreads();
        float px[TI], py[TI], pz[TI];
#pragma unroll
        for (int k = 0; k < TI; ++k) px[k] = py[k] = pz[k] = 0.f;
        if (!PLAIN && far)
            grav_tile<true, TI, PACKED, false, UNIFORM>(sh_hi, sh_lo, j0, ii, hx, hy, hz, lx, ly, lz, px, py, pz);
        else if ((j0 < ib0 + TI * GB) && (j0 + GB > ib0))
            grav_tile<PLAIN, TI, PACKED, true, UNIFORM>(sh_hi, sh_lo, j0, ii, hx, hy, hz, lx, ly, lz, px, py, pz);
        else
            grav_tile<PLAIN, TI, PACKED, false, UNIFORM>(sh_hi, sh_lo, j0, ii, hx, hy, hz, lx, ly, lz, px, py, pz);
#pragma unroll
        for (int k = 0; k < TI; ++k) {
            ax[k].add(px[k]);
            ay[k].add(py[k]);
            az[k].add(pz[k]);
        }
    }
#pragma unroll
    for (int k = 0; k < TI; ++k) {
        if (ii[k] < n) {
            double* p = part + ((int64_t)jc * n + ii[k]) * 3;
            p[0] = ax[k].value();
            p[1] = ay[k].value();
            p[2] = az[k].value();
        }
    }
}

typedef void (*grav_kernel_t)(const float4*, const float4*, int64_t, int64_t, int, double*, const float4*, float);

// Kernel variants: bodies per thread (TI) x packed FP32x2; index
// 0: TI=2 scalar, 1: TI=2 packed, 2: TI=4 scalar, 3: TI=4 packed, 4: TI=1 scalar.
// uniform (equal masses) selects the packed forms without m_j in the loop.
static grav_kernel_t grav_variant(bool plain, int v, bool uniform)
{
    switch (v) {
    case 0: return plain ? k_gravity<true, 2, false, false> : k_gravity<false, 2, false, false>;
    case 2: return plain ? k_gravity<true, 4, false, false> : k_gravity<false, 4, false, false>;
    case 3:
        if (uniform) return plain ? k_gravity<true, 4, true, true> : k_gravity<false, 4, true, true>;
        return plain ? k_gravity<true, 4, true, false> : k_gravity<false, 4, true, false>;
    case 4: return plain ? k_gravity<true, 1, false, false> : k_gravity<false, 1, false, false>;
    default:
        if (uniform) return plain ? k_gravity<true, 2, true, true> : k_gravity<false, 2, true, true>;
        return plain ? k_gravity<true, 2, true, false> : k_gravity<false, 2, true, false>;
    }
}
static bool grav_variant_packed(int v) { return v == 1 || v == 3 || v < 0 || v > 4; }
static int grav_ti(int v) { return v == 2 || v == 3 ? 4 : (v == 4 ? 1 : 2); }

// a_i = -G sum_chunks partial_i (fixed chunk order); with a permutation the
// partials are in sorted order and body perm[s] receives slot s
__global__ void k_gravity_reduce(const double* __restrict__ part, int64_t n, int jchunks, double G,
                                 double* __restrict__ A, unsigned* status, const int* __restrict__ perm)
{
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < 3 * n; e += (int64_t)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int c = 0; c < jchunks; ++c) s += part[(int64_t)c * 3 * n + e];
        double a = -G * s;
        if (!finite64(a)) status_set(status, ST_NONFINITE);
        const int64_t slot = e / 3;
        A[perm ? 3 * (int64_t)perm[slot] + (e - 3 * slot) : e] = a;
    }
}

// Morton order of the bodies: 21 bits per dimension of the position in
// [-S, S]^3 (clamped), interleaved (x in the top bit of each triple). The
// fine grid keeps a concentrated core ordered when a few bodies lie far out.
__device__ __forceinline__ unsigned long long spread3(unsigned long long v)
{
    v &= 0x1fffffull;
    v = (v | (v << 32)) & 0x1f00000000ffffull;
    v = (v | (v << 16)) & 0x1f0000ff0000ffull;
    v = (v | (v << 8)) & 0x100f00f00f00f00full;
    v = (v | (v << 4)) & 0x10c30c30c30c30c3ull;
    v = (v | (v << 2)) & 0x1249249249249249ull;
    return v;
}

// Largest |coordinate| of the finite positions, rounded up to FP32, as the
// bits of a non-negative float (which order like unsigned integers): the
// half-width of the Morton cube. *ext must be 0 before the launch.
__global__ void k_grav_extent(const double* __restrict__ X, int64_t m, unsigned* ext)
{
    float v = 0.f;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < m; e += (int64_t)gridDim.x * blockDim.x) {
        const double a = fabs(X[e]);
        if (isfinite(a)) v = fmaxf(v, __double2float_ru(a));
    }
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) atomicMax(ext, __float_as_uint(v));
}

__global__ void k_grav_keys(const double* __restrict__ X, int64_t n, const unsigned* __restrict__ ext,
                            unsigned long long* keys, int* vals)
{
    const double cells = 2097152.0;  // 2^21
    const double S = (double)__uint_as_float(*ext) * 1.0001;
    const double inv2S = S > 0.0 && isfinite(S) ? 0.5 / S : 0.5;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        unsigned long long q[3];
        for (int k = 0; k < 3; ++k) {
            double t = (X[3 * i + k] * inv2S + 0.5) * cells;
            t = t < 0.0 ? 0.0 : (t > cells - 1.0 ? cells - 1.0 : t);
            q[k] = isfinite(t) ? (unsigned long long)t : 0ull;
        }
        keys[i] = (spread3(q[0]) << 2) | (spread3(q[1]) << 1) | spread3(q[2]);
        vals[i] = (int)i;
    }
}

// split positions and masses in sorted order (slot s holds body perm[s])
__global__ void k_grav_pack_sorted(const double* __restrict__ X, const double* __restrict__ mass,
                                   const int* __restrict__ perm, int64_t n, float4* phi, float4* plo)
{
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n; s += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = perm[s];
        float h[3], l[3];
        for (int k = 0; k < 3; ++k) {
            const double p = X[3 * i + k];
            h[k] = (float)p;
            l[k] = (float)(p - (double)h[k]);
        }
        phi[s] = make_float4(h[0], h[1], h[2], (float)mass[i]);
        plo[s] = make_float4(l[0], l[1], l[2], 0.f);
    }
}

// per 128-body tile over its real bodies: box min (x, y, z, largest |r|) and
// box max (x, y, z, smallest |r|) (an empty tile gets an inverted box)
__global__ void __launch_bounds__(GB) k_grav_boxes(const float4* __restrict__ phi, int64_t n, float4* box)
{
    const int64_t s = blockIdx.x * (int64_t)GB + threadIdx.x;
    float v[8];  // minima of x, y, z, -x, -y, -z, |r|, -|r|
    if (s < n) {
        const float4 h = phi[s];
        const float r = sqrtf(h.x * h.x + h.y * h.y + h.z * h.z);
        v[0] = h.x; v[1] = h.y; v[2] = h.z;
        v[3] = -h.x; v[4] = -h.y; v[5] = -h.z;
        v[6] = r; v[7] = -r;
    } else {
        for (int k = 0; k < 8; ++k) v[k] = INFINITY;
    }
    for (int o = 16; o > 0; o >>= 1)
        for (int k = 0; k < 8; ++k) v[k] = fminf(v[k], __shfl_xor_sync(0xffffffffu, v[k], o));
    __shared__ float red[GB / 32][8];
    if ((threadIdx.x & 31) == 0)
        for (int k = 0; k < 8; ++k) red[threadIdx.x / 32][k] = v[k];
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < GB / 32; ++w)
            for (int k = 0; k < 8; ++k) v[k] = fminf(v[k], red[w][k]);
        box[2 * blockIdx.x] = make_float4(v[0], v[1], v[2], -v[7]);
        box[2 * blockIdx.x + 1] = make_float4(-v[3], -v[4], -v[5], v[6]);
    }
}

// Number of j-chunks: the smallest that makes (i-blocks x chunks) fill the
// resident block slots (SMs x blocks per SM) in near-whole waves.
static int plan_gravity(nbg_ctx* c, int64_t npad)
{
    int dev = c->device, sms = 0, occ = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, grav_variant(c->d.grav_plain, c->grav_variant, c->grav_uniform),
                                                  GB, 0);
    if (sms < 1) sms = 1;
    if (occ < 1) occ = 1;
    const double slots = (double)sms * occ;
    const int64_t ib = npad / (grav_ti(c->grav_variant) * GB);
    const int64_t ntile = npad / GB;
    int best = 1;
    double best_eff = -1.0;
    for (int J = 1; J <= 64 && J <= ntile; ++J) {
        double waves = (double)(ib * J) / slots;
        // whole-wave efficiency, with chunks of ceil(ntile/J) vs ntile/J tiles
        double eff = waves / ceil(waves) * ((double)ntile / J) / (double)((ntile + J - 1) / J);
        if (eff > best_eff + 0.005) {
            best_eff = eff;
            best = J;
        }
        if (eff >= 0.97) break;
    }
    return best;
}

// Launch the gravity kernel and the chunk reduction into s.a_new. The
// partials (grav_chunks * n * 3 doubles) live in c->grav_part.
int launch_gravity(nbg_ctx* c, const StateView& s)
{
    int64_t units = (c->npad / (grav_ti(c->grav_variant) * GB)) * c->grav_chunks;
    const bool uniform = c->grav_uniform && grav_variant_packed(c->grav_variant);
    grav_kernel_t kern = grav_variant(c->d.grav_plain, c->grav_variant, uniform);
    const int* perm = nullptr;
    if (c->grav_sort) {
        // Morton sort (every 8th evaluation: the bodies move little in
        // between), sorted split positions, tile boxes
        if (!c->grav_perm_valid || c->grav_evals % 8 == 0) {
            cudaError_t me = cudaMemsetAsync(c->grav_extent, 0, sizeof(unsigned), c->stream);
            if (me != cudaSuccess) return cuda_fail(c, me, "gravity extent clear");
            k_grav_extent<<<2 * c->sms, 256, 0, c->stream>>>(s.x, 3 * c->n, c->grav_extent);
            NBG_LAUNCH_CHECK(c, "k_grav_extent");
            k_grav_keys<<<grid_for(c->n, 256), 256, 0, c->stream>>>(s.x, c->n, c->grav_extent, c->grav_keys[0],
                                                                     c->grav_vals[0]);
            NBG_LAUNCH_CHECK(c, "k_grav_keys");
            size_t bytes = c->grav_sort_bytes;
            cudaError_t e = cub::DeviceRadixSort::SortPairs(c->grav_sort_tmp, bytes, c->grav_keys[0], c->grav_keys[1],
                                                            c->grav_vals[0], c->grav_vals[1], (int)c->n, 0, 63,
                                                            c->stream);
            if (e != cudaSuccess) return cuda_fail(c, e, "gravity Morton sort");
            c->launches += 8;  // the sort's own passes
            c->grav_perm_valid = true;
        }
        ++c->grav_evals;
        perm = c->grav_vals[1];
        k_grav_pack_sorted<<<grid_for(c->n, 256), 256, 0, c->stream>>>(s.x, c->d.mass, perm, c->n, c->d.phi,
                                                                          c->d.plo);
        NBG_LAUNCH_CHECK(c, "k_grav_pack_sorted");
        k_grav_boxes<<<(unsigned)(c->npad / GB), GB, 0, c->stream>>>(c->d.phi, c->n, c->grav_box);
        NBG_LAUNCH_CHECK(c, "k_grav_boxes");
    }
    prof_begin(c);
    kern<<<(unsigned)units, GB, 0, c->stream>>>(c->d.phi, c->d.plo, c->n, c->npad, c->grav_chunks, c->grav_part,
                                                c->grav_sort ? c->grav_box : nullptr, c->grav_far2);
    prof_end(c);
    NBG_LAUNCH_CHECK(c, "k_gravity");
    k_gravity_reduce<<<grid_for(3 * c->n, 256), 256, 0, c->stream>>>(c->grav_part, c->n, c->grav_chunks,
                                                                      uniform ? c->d.G * c->grav_m0 : c->d.G,
                                                                      s.a_new, c->d.status, perm);
    NBG_LAUNCH_CHECK(c, "k_gravity_reduce");
    return NBG_OK;
}

// scratch of the Morton sort (keys, values and cub's temporary storage) and
// the tile boxes
size_t gravity_sort_bytes(int64_t n)
{
    size_t bytes = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, bytes, (unsigned long long*)nullptr, (unsigned long long*)nullptr,
                                    (int*)nullptr, (int*)nullptr, (int)n, 0, 63);
    return bytes;
}

int gravity_plan_chunks(nbg_ctx* c, int64_t npad) { return plan_gravity(c, npad); }

// ---------------------------------------------------------------------
// generic all-pairs kernel
// ---------------------------------------------------------------------
#define AT 128

__global__ void __launch_bounds__(AT) k_allpairs(Dev d, StateView s)
{
    __shared__ float4 sh_hi[AT];
    __shared__ float4 sh_lo[AT];
    __shared__ float sh_m[AT];
    __shared__ float3 sh_mm[AT];
    const int64_t i = blockIdx.x * (int64_t)AT + threadIdx.x;
    const bool active = i < d.n;
    const int64_t ii = active ? i : 0;
    const RepDev& R = d.reps[0];
    const PairK K(R);
    float4 hi_i = d.phi[ii], lo_i = d.plo[ii];
    float kqi = (d.pots & NBG_POT_EL) ? (float)(d.el_k_d * d.charge[ii]) : 0.0f;
    float3 mi = make_float3(0.f, 0.f, 0.f);
    if (d.pots & NBG_POT_MAG) mi = make_float3((float)d.dipole[3 * ii], (float)d.dipole[3 * ii + 1], (float)d.dipole[3 * ii + 2]);
    Acc2 fx{0.f, 0.f}, fy{0.f, 0.f}, fz{0.f, 0.f};   // LJ + electrostatic force
    Acc2 gx{0.f, 0.f}, gy{0.f, 0.f}, gz{0.f, 0.f};   // gravity sum m_j r / r^3
    Acc2 mx{0.f, 0.f}, my{0.f, 0.f}, mz{0.f, 0.f};   // dipole sum
    bool range_err = false;
    const bool cutpots = (d.pots & (NBG_POT_LJ | NBG_POT_EL)) != 0;
    for (int64_t t = 0; t < d.n; t += AT) {
        __syncthreads();
        int64_t j = t + threadIdx.x;
        if (j < d.n) {
            sh_hi[threadIdx.x] = d.phi[j];
            sh_lo[threadIdx.x] = d.plo[j];
            sh_m[threadIdx.x] = (float)d.mass[j];
            if (d.pots & NBG_POT_MAG)
                sh_mm[threadIdx.x] = make_float3((float)d.dipole[3 * j], (float)d.dipole[3 * j + 1], (float)d.dipole[3 * j + 2]);
        }
        __syncthreads();
        int m = (int)((d.n - t) < AT ? (d.n - t) : AT);
        float px = 0.f, py = 0.f, pz = 0.f, qx = 0.f, qy = 0.f, qz = 0.f, wx = 0.f, wy = 0.f, wz = 0.f;
        for (int k = 0; k < m; ++k) {
            int64_t jg = t + k;
            if (jg == ii) continue;
            float4 hj = sh_hi[k], lj = sh_lo[k];
            if (cutpots) {
                PairOut o = pair_cutoff(d, R, K, ii, jg, hi_i, lo_i, hj, lj, kqi, s.x);
                range_err |= o.range_err;
                px += o.fx;
                py += o.fy;
                pz += o.fz;
            }
            if (d.pots & (NBG_POT_GRAV | NBG_POT_MAG)) {
                // plain differences: gravity and dipoles ignore the boundary
                float3 dr = split_diff(hi_i, lo_i, hj, lj, false, R);
                float r2 = fmaf(dr.x, dr.x, fmaf(dr.y, dr.y, dr.z * dr.z));
                float ri = rsqrtf(r2);
                if (d.pots & NBG_POT_GRAV) {
                    float sg = sh_m[k] * ri * ri * ri;
                    qx = fmaf(sg, dr.x, qx);
                    qy = fmaf(sg, dr.y, qy);
                    qz = fmaf(sg, dr.z, qz);
                }
                if (d.pots & NBG_POT_MAG) {
                    // (mi (mj.r) + mj (mi.r) + r (mi.mj) - 5 r (mi.r)(mj.r)) / |r|^4, r unit
                    float3 u = make_float3(dr.x * ri, dr.y * ri, dr.z * ri);
                    float3 mj = sh_mm[k];
                    float mir = mi.x * u.x + mi.y * u.y + mi.z * u.z;
                    float mjr = mj.x * u.x + mj.y * u.y + mj.z * u.z;
                    float mimj = mi.x * mj.x + mi.y * mj.y + mi.z * mj.z;
                    float inv4 = (ri * ri) * (ri * ri);
                    wx += (mi.x * mjr + mj.x * mir + u.x * mimj - 5.0f * u.x * mir * mjr) * inv4;
                    wy += (mi.y * mjr + mj.y * mir + u.y * mimj - 5.0f * u.y * mir * mjr) * inv4;
                    wz += (mi.z * mjr + mj.z * mir + u.z * mimj - 5.0f * u.z * mir * mjr) * inv4;
                }
            }
        }
        fx.add(px); fy.add(py); fz.add(pz);
        gx.add(qx); gy.add(qy); gz.add(qz);
        mx.add(wx); my.add(wy); mz.add(wz);
    }
    if (range_err) status_set(d.status, ST_RANGE);
    if (!active) return;
    const double im = d.inv_mass[i];
    double a[3] = {fx.value() * im, fy.value() * im, fz.value() * im};
    if (d.pots & NBG_POT_GRAV) {
        a[0] += -d.G * gx.value();
        a[1] += -d.G * gy.value();
        a[2] += -d.G * gz.value();
    }
    if (d.pots & NBG_POT_MAG) {
        double cm = 3.0 * d.mu4pi / d.mass[i];
        a[0] += cm * mx.value();
        a[1] += cm * my.value();
        a[2] += cm * mz.value();
    }
    for (int k = 0; k < 3; ++k) {
        if (!finite64(a[k])) status_set(d.status, ST_NONFINITE);
        s.a_new[3 * i + k] = a[k];
    }
}

int launch_allpairs(nbg_ctx* c, const StateView& s)
{
    prof_begin(c);
    k_allpairs<<<grid_for(c->n, AT), AT, 0, c->stream>>>(c->d, s);
    prof_end(c);
    NBG_LAUNCH_CHECK(c, "k_allpairs");
    return NBG_OK;
}

// ---------------------------------------------------------------------
// Verlet-list force kernels
// ---------------------------------------------------------------------
// Thread per atom over a column-major list (coalesced across the atoms of a
// warp): for large systems, where every SM has thousands of atoms.
__global__ void __launch_bounds__(128) k_force_list(Dev d, StateView s)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < d.n; i += (int64_t)gridDim.x * blockDim.x) {
        const RepDev& R = d.reps[d.rep_of[i]];
        const PairK K(R);
        const float4 hi_i = d.phi[i], lo_i = d.plo[i];
        const float kqi = (d.pots & NBG_POT_EL) ? (float)(d.el_k_d * d.charge[i]) : 0.0f;
        const int cnt = d.nbr_count[i];
        Acc2 fx{0.f, 0.f}, fy{0.f, 0.f}, fz{0.f, 0.f};
        float px = 0.f, py = 0.f, pz = 0.f;
        bool range_err = false;
        const int* nl = d.nbr + i * d.nbr_istride;
        // the next neighbour's index and split position are loaded one entry
        // ahead, so that their gathers overlap this pair's arithmetic
        int jn = 0;
        float4 hn = make_float4(0.f, 0.f, 0.f, 0.f), ln = hn;
        if (cnt > 0) {
            jn = dbg_index(__ldg(nl), d.n, (int)i, d.status);
            hn = __ldg(&d.phi[jn]);
            ln = __ldg(&d.plo[jn]);
        }
        for (int k = 0; k < cnt; ++k) {
            const int j = jn;
            const float4 hj = hn, lj = ln;
            if (k + 1 < cnt) {
                jn = dbg_index(__ldg(nl + (int64_t)(k + 1) * d.nbr_kstride), d.n, (int)i, d.status);
                hn = __ldg(&d.phi[jn]);
                ln = __ldg(&d.plo[jn]);
            }
            PairOut o = pair_cutoff(d, R, K, i, j, hi_i, lo_i, hj, lj, kqi, s.x);
            range_err |= o.range_err;
            px += o.fx;
            py += o.fy;
            pz += o.fz;
            if ((k & 31) == 31) {
                fx.add(px); fy.add(py); fz.add(pz);
                px = py = pz = 0.f;
            }
        }
        fx.add(px); fy.add(py); fz.add(pz);
        if (range_err) status_set(d.status, ST_RANGE);
        const double im = d.inv_mass[i];
        double a0 = fx.value() * im, a1 = fy.value() * im, a2 = fz.value() * im;
        if (!finite64(a0) || !finite64(a1) || !finite64(a2)) status_set(d.status, ST_NONFINITE);
        s.a_new[3 * i] = a0;
        s.a_new[3 * i + 1] = a1;
        s.a_new[3 * i + 2] = a2;
    }
}

// (h, e) += the partner lane's (h, e), h by TwoSum with its error into e
__device__ __forceinline__ void lane_join(float& h, float& e, int o, int width)
{
    const float h2 = __shfl_xor_sync(0xffffffffu, h, o, width);
    const float e2 = __shfl_xor_sync(0xffffffffu, e, o, width);
    float sum, err;
    two_sum(h, h2, sum, err);
    h = sum;
    e = __fadd_rn(__fadd_rn(e, e2), err);
}

// LPA lanes per atom over a row-major list: the group reads its atom's
// entries coalesced, each lane keeps an FP32 partial of every LPA-th entry,
// and the partials are joined by a compensated FP32 xor butterfly of shuffles
// (a fixed order: deterministic); one FP64 multiply by 1/m per component
// gives the acceleration. For small systems, where one atom per thread
// leaves the GPU waiting on memory latency.
template <int LPA>
__global__ void __launch_bounds__(256) k_force_list_lanes(Dev d, StateView s)
{
    // one atom per group of LPA lanes; groups past n keep running (with no
    // entries) so that every lane of the warp takes part in the shuffles
    const int lane = threadIdx.x % LPA;
    const int64_t i = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / LPA;
    const bool active = i < d.n;
    const int64_t ia = active ? i : 0;
    const RepDev& R = d.reps[d.rep_of[ia]];
    const float4 hi_i = d.phi[ia], lo_i = d.plo[ia];
    const float kqi = (d.pots & NBG_POT_EL) ? (float)(d.el_k_d * d.charge[ia]) : 0.0f;
    const int cnt = active ? d.nbr_count[ia] : 0;
    float px = 0.f, py = 0.f, pz = 0.f;
    bool range_err = false;
    const int* nl = d.nbr + ia * d.nbr_istride;
    // the pair constants in registers pay off for the short lists of 4-lane
    // groups (LJ ensembles); longer lists keep fewer registers (more warps)
    auto pair_loop = [&](const auto& K) {
        for (int k = lane; k < cnt; k += LPA) {
            int j = dbg_index(__ldg(nl + k), d.n, (int)ia, d.status);
            float4 hj = __ldg(&d.phi[j]), lj = __ldg(&d.plo[j]);
            PairOut o = pair_cutoff(d, R, K, ia, j, hi_i, lo_i, hj, lj, kqi, s.x);
            range_err |= o.range_err;
            px += o.fx;
            py += o.fy;
            pz += o.fz;
        }
    };
    if constexpr (LPA <= 4) pair_loop(PairK(R));
    else pair_loop(R);
    // join the lanes' partials: compensated FP32 butterfly (TwoSum; every
    // lane ends with the same value, whatever the order of its operands)
    float ex = 0.f, ey = 0.f, ez = 0.f;
#pragma unroll
    for (int o = LPA / 2; o > 0; o >>= 1) {
        lane_join(px, ex, o, LPA);
        lane_join(py, ey, o, LPA);
        lane_join(pz, ez, o, LPA);
    }
    if (range_err) status_set(d.status, ST_RANGE);
    if (active && lane == 0) {
        const double im = d.inv_mass[i];
        const double a0 = ((double)px + (double)ex) * im, a1 = ((double)py + (double)ey) * im,
                     a2 = ((double)pz + (double)ez) * im;
        if (!finite64(a0) || !finite64(a1) || !finite64(a2)) status_set(d.status, ST_NONFINITE);
        s.a_new[3 * i] = a0;
        s.a_new[3 * i + 1] = a1;
        s.a_new[3 * i + 2] = a2;
    }
}

int launch_force_list(nbg_ctx* c, const StateView& s)
{
    if (c->fx_ready) return launch_force_fx(c, s);
    const int lpa = c->list_lpa;
    prof_begin(c);
    if (lpa <= 1) {
        k_force_list<<<grid_for(c->n, 128), 128, 0, c->stream>>>(c->d, s);
    } else {
        const int per_block = 256 / lpa;  // one atom per group, whole groups per block
        int grid = (int)((c->n + per_block - 1) / per_block);
        if (lpa == 4) k_force_list_lanes<4><<<grid, 256, 0, c->stream>>>(c->d, s);
        else if (lpa == 8) k_force_list_lanes<8><<<grid, 256, 0, c->stream>>>(c->d, s);
        else if (lpa == 16) k_force_list_lanes<16><<<grid, 256, 0, c->stream>>>(c->d, s);
        else k_force_list_lanes<32><<<grid, 256, 0, c->stream>>>(c->d, s);
    }
    prof_end(c);
    NBG_LAUNCH_CHECK(c, "k_force_list");
    return NBG_OK;
}

// ---------------------------------------------------------------------
// SPC/Fw bonded terms (FP64), one thread per molecule (O, H1, H2)
// ---------------------------------------------------------------------
__device__ __forceinline__ void cross3f(const float* a, const float* b, float* c)
{
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

__device__ __forceinline__ float norm3f(const float* a) { return sqrtf(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]); }

// Bonds and angle of one molecule. The intramolecular differences are taken
// in FP64 from the unwrapped positions and rounded once to FP32 (relative
// error 2^-24); the terms themselves are FP32, like the pair forces (the bond
// stretch r - rOH and the angle offset then carry ~1e-6 relative error). The
// accelerations are added to a_new in FP64.
__global__ void k_bonded(Dev d, StateView s)
{
    int64_t nm = d.n / 3;
    const float rOH = (float)d.rOH, kb = (float)d.kbond, ka = (float)d.kangle, a0 = (float)d.aHOH;
    for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < nm; m += (int64_t)gridDim.x * blockDim.x) {
        int64_t o = 3 * m, h1 = o + 1, h2 = o + 2;
        const double* X = s.x;
        float r1[3], r2[3];  // H1 - O, H2 - O
        for (int k = 0; k < 3; ++k) {
            r1[k] = (float)(X[3 * h1 + k] - X[3 * o + k]);
            r2[k] = (float)(X[3 * h2 + k] - X[3 * o + k]);
        }
        // bonds (harmonic_bond_potential_acceleration!, :367-393): on O from
        // bond O-H, -(r - rOH) k / r (r_O - r_H); on H the exact negative.
        float fO[3] = {0.f, 0.f, 0.f}, fH1[3], fH2[3];
        const float* hs[2] = {r1, r2};
        float* fh[2] = {fH1, fH2};
        for (int b = 0; b < 2; ++b) {
            float r = norm3f(hs[b]);
            float factor = -(r - rOH) * kb / r;
            for (int k = 0; k < 3; ++k) {
                float f = factor * -hs[b][k];  // rij = r_O - r_H
                fO[k] += f;
                fh[b][k] = -f;
            }
        }
        // angle H1-O-H2 (valence_angle_potential_acceleration!, :395-433), a=H1, b=O, c=H2
        float rcb[3] = {-r2[0], -r2[1], -r2[2]}, x[3], pa[3], pc[3];
        cross3f(r1, r2, x);
        cross3f(r1, x, pa);
        cross3f(rcb, x, pc);
        float npa = norm3f(pa), npc = norm3f(pc);
        float nba = norm3f(r1), nbc = norm3f(r2);
        float cosine = (r1[0] * r2[0] + r1[1] * r2[1] + r1[2] * r2[2]) / (nba * nbc);
        cosine = fminf(1.0f, fmaxf(-1.0f, cosine));
        float force = -ka * (acosf(cosine) - a0);
        float sa = force / (npa * nba), sc = force / (npc * nbc);
        const double iO = d.inv_mass[o], iH1 = d.inv_mass[h1], iH2 = d.inv_mass[h2];
        for (int k = 0; k < 3; ++k) {
            float fa = pa[k] * sa;
            float fc = pc[k] * sc;
            float fb = -(fa + fc);
            s.a_new[3 * o + k] += (double)(fO[k] + fb) * iO;
            s.a_new[3 * h1 + k] += (double)(fH1[k] + fa) * iH1;
            s.a_new[3 * h2 + k] += (double)(fH2[k] + fc) * iH2;
        }
    }
}

int launch_bonded(nbg_ctx* c, const StateView& s)
{
    k_bonded<<<grid_for(c->n / 3, 64), 64, 0, c->stream>>>(c->d, s);
    NBG_LAUNCH_CHECK(c, "k_bonded");
    return NBG_OK;
}

// ---------------------------------------------------------------------
// Raw launcher of the gravity kernel (default form) and its chunk reduction
// on caller-provided buffers, for entry points that own their scratch.
// ---------------------------------------------------------------------
int gravity_raw_chunks(int device, int64_t npad, int max_chunks)
{
    int sms = 0, occ = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_gravity<false, 2, true, false>, GB, 0);
    if (sms < 1) sms = 1;
    if (occ < 1) occ = 1;
    const double slots = (double)sms * occ;
    const int64_t ib = npad / (2 * GB);
    const int64_t ntile = npad / GB;
    int best = 1;
    double best_eff = -1.0;
    for (int J = 1; J <= max_chunks && J <= ntile; ++J) {
        double waves = (double)(ib * J) / slots;
        double eff = waves / ceil(waves) * ((double)ntile / J) / (double)((ntile + J - 1) / J);
        if (eff > best_eff + 0.005) {
            best_eff = eff;
            best = J;
        }
    }
    return best;
}

cudaError_t gravity_raw_launch(const float4* phi, const float4* plo, int64_t n, int64_t npad, int jchunks,
                               double* part, double G, double* a, unsigned* status, cudaStream_t stream)
{
    int64_t units = (npad / (2 * GB)) * jchunks;
    k_gravity<false, 2, true, false><<<(unsigned)units, GB, 0, stream>>>(phi, plo, n, npad, jchunks, part, nullptr, 0.f);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_gravity_reduce<<<grid_for(3 * n, 256), 256, 0, stream>>>(part, n, jchunks, G, a, status, nullptr);
    return cudaGetLastError();
}
