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
