// fx_pair.cuh - one pair on fixed-point box coordinates: the wrapped
// difference, the FP32 classification against the cutoffs and its FP64
// fallback. Shared by the list force kernel (k_force_fx.cu) and the
// pair-set export (k_energy.cu), so that the exported set is the set the
// forces count.
#pragma once

#include "nbg_internal.cuh"

// Difference of two fixed-point coordinates: the wrapping 32-bit difference
// read as int32 (the minimum image into [-L/2, L/2)), rounded to FP32 once.
__device__ __forceinline__ float fx_diff(unsigned a, unsigned b) { return (float)(int)(a - b); }

__device__ __forceinline__ float fx_r2(const uint4& qi, const uint4& qj, float& dx, float& dy, float& dz)
{
    dx = fx_diff(qi.x, qj.x);
    dy = fx_diff(qi.y, qj.y);
    dz = fx_diff(qi.z, qj.z);
    return __fmaf_rn(dx, dx, __fmaf_rn(dy, dy, __fmul_rn(dz, dz)));
}

// j % 3 == 0 for 0 <= j < 2^31 (divisibility by the inverse of 3 mod 2^32):
// the water oxygens, the only LJ sites of WaterSPCFw
__device__ __forceinline__ bool fx_oxygen(int j) { return (unsigned)j * 0xAAAAAAABu <= 0x55555555u; }

// Membership of a pair with box-unit r^2 in the LJ (lp: an LJ pair) and EL
// (ep) cutoffs where FP32 decides it, and amb where it does not (within the
// relative band of a cutoff, or past the half-box band).
__device__ __forceinline__ void fx_classify(float r2, bool lp, bool ep, float lj_lo, float lj_hi, float el_lo,
                                            float el_hi, bool& lj_in, bool& el_in, bool& amb)
{
    lj_in = lp && r2 < lj_lo;
    el_in = ep && r2 < el_lo;
    amb = (lp && !lj_in && r2 < lj_hi) || (ep && !el_in && r2 < el_hi);
}

// The pair decided again in the reference's FP64 arithmetic on the unwrapped
// positions (boundary_conditions.jl:138-165, basic_potentials.jl:253-258,
// 288-292): membership, and the FP64 difference in box units.
struct FxPair {
    float dx, dy, dz, r2;
    int lj_in, el_in, range_err;
};

static __device__ __noinline__ FxPair fx_pair_fallback(const Dev d, const double* X, int64_t i, int64_t j,
                                                       int lj_pair, int el_pair)
{
    FxPair o{0.f, 0.f, 0.f, 1.0f, 0, 0, 0};
    const RepDev& R = d.reps[d.rep_of[i]];
    Dist64 q;
    if (!distance64<false>(X + 3 * i, X + 3 * j, NBG_BC_CUBIC, R, q)) {
        o.range_err = 1;
        return o;
    }
    o.lj_in = lj_pair && (q.r2 < d.lj_R2);
    o.el_in = el_pair && (q.r2 < d.el_R2);
    const double s = R.fx_scale;
    o.dx = (float)(q.x * s);
    o.dy = (float)(q.y * s);
    o.dz = (float)(q.z * s);
    o.r2 = __fmaf_rn(o.dx, o.dx, __fmaf_rn(o.dy, o.dy, __fmul_rn(o.dz, o.dz)));
    return o;
}

// Potential kinds of the fixed-point pair kernels (compile-time forms).
enum { FX_LJ = 1, FX_EL = 2, FX_LJEL = 3, FX_WATER = 4 };

// (h, e) += the partner lane's (h, e): TwoSum of the h parts, errors into e
__device__ __forceinline__ void fx_join(float& h, float& e, int o, int width)
{
    const float h2 = __shfl_xor_sync(0xffffffffu, h, o, width);
    const float e2 = __shfl_xor_sync(0xffffffffu, e, o, width);
    float sum, err;
    two_sum(h, h2, sum, err);
    h = sum;
    e = __fadd_rn(__fadd_rn(e, e2), err);
}

// One packed pair step (entries k0 and k0 + LPA of atom row a) of the
// fixed-point kernels: classification, FP64 fallback, LJ and reaction-field
// factors in the units of the LJ sum, accumulated into (px, py, pz). An
// entry with v0 / v1 false adds exactly zero (its partner must be a valid
// index, e.g. the atom itself).
template <int POT>
__device__ __forceinline__ void fx_pair2(const Dev& d, const double* X, int64_t ia, bool lj_i, float kqi,
                                         const uint4& qi, int j0, int j1, bool v0, bool v1, const uint4& q0,
                                         const uint4& q1, float lj_lo, float lj_hi, float el_lo, float el_hi,
                                         float sig2h, float sig2l, float krf, float2& px, float2& py, float2& pz,
                                         bool& range_err)
{
    constexpr bool HAS_LJ = POT == FX_LJ || POT == FX_LJEL || POT == FX_WATER;
    constexpr bool HAS_EL = POT == FX_EL || POT == FX_LJEL || POT == FX_WATER;
    float2 dx = make_float2(fx_diff(qi.x, q0.x), fx_diff(qi.x, q1.x));
    float2 dy = make_float2(fx_diff(qi.y, q0.y), fx_diff(qi.y, q1.y));
    float2 dz = make_float2(fx_diff(qi.z, q0.z), fx_diff(qi.z, q1.z));
    float2 r2 = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __fmul2_rn(dz, dz)));
    const bool lp0 = HAS_LJ && v0 && lj_i && (POT != FX_WATER || fx_oxygen(j0));
    const bool lp1 = HAS_LJ && v1 && lj_i && (POT != FX_WATER || fx_oxygen(j1));
    const bool ep0 = HAS_EL && v0, ep1 = HAS_EL && v1;
    bool lj0, lj1, el0, el1b, amb0, amb1;
    fx_classify(r2.x, lp0, ep0, lj_lo, lj_hi, el_lo, el_hi, lj0, el0, amb0);
    fx_classify(r2.y, lp1, ep1, lj_lo, lj_hi, el_lo, el_hi, lj1, el1b, amb1);
    if (amb0 | amb1) {
        if (amb0) {
            const FxPair o = fx_pair_fallback(d, X, ia, j0, lp0, ep0);
            lj0 = o.lj_in;
            el0 = o.el_in;
            dx.x = o.dx, dy.x = o.dy, dz.x = o.dz, r2.x = o.r2;
            range_err |= o.range_err != 0;
        }
        if (amb1) {
            const FxPair o = fx_pair_fallback(d, X, ia, j1, lp1, ep1);
            lj1 = o.lj_in;
            el1b = o.el_in;
            dx.y = o.dx, dy.y = o.dy, dz.y = o.dz, r2.y = o.r2;
            range_err |= o.range_err != 0;
        }
    }
    const bool in0 = lj0 || el0, in1 = lj1 || el1b;
    r2 = make_float2(in0 ? r2.x : 1.0f, in1 ? r2.y : 1.0f);
    float2 f = make_float2(0.f, 0.f);
    if (HAS_LJ) {
        const float2 ri = make_float2(__fdividef(1.0f, r2.x), __fdividef(1.0f, r2.y));
        const float2 s2 = __ffma2_rn(make_float2(sig2h, sig2h), ri, __fmul2_rn(make_float2(sig2l, sig2l), ri));
        const float2 s6 = __fmul2_rn(__fmul2_rn(s2, s2), s2);
        const float2 fl =
            __fmul2_rn(__fmul2_rn(__ffma2_rn(make_float2(2.f, 2.f), s6, make_float2(-1.f, -1.f)), s6), ri);
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

