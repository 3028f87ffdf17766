// k_learned.cu - the learned short-range force model of SPC/Fw water and its
// training (no reference counterpart: an engine feature). The definitions are
// the ones oracle/learned.py restates in FP64:
//
//  descriptor of atom i over atoms j of other molecules with r < ML_RD:
//    radial   G[s][k] = sum_{j in s} g_k(r) fc(r), Gaussians of width w at
//             mu_k = ML_R0 + k w (24 per neighbour species s)
//    angular  p[s][a] = sum psi_a(r) rhat, Q[s][a] = sum psi_a (rhat rhat^T - I/3),
//             psi_a = fc(r) exp(-r^2 / (2 rho_a^2)), invariants |p|^2, |Q|_F^2
//    D = [G_O(24), G_H(24), A1_O(4), A1_H(4), A2_O(4), A2_H(4)] (64)
//  per-species MLP 64 -> 128 -> 128 -> 1 (tanh): E_i = sdE (a2 . w3 + b3) + muE
//    on the standardised input x = (D - muD) / sdD.
//  short-range target: E_i = 1/2 sum_j phi(r) S(r), phi = LJ (O-O) +
//    k q_i q_j erfc(alpha r) / r (the real-space part of an Ewald-type
//    split), S a C2 smoothstep from 1 at ML_RS to 0 at ML_RD. The screening
//    keeps the switched region's forces small, so that the remainder (exact
//    non-bonded force minus this part) varies slowly enough for the outer
//    step of r-RESPA.
//
// Short lists hold, per atom, the long-list atoms within ML_RD + skin split by
// species (O from the front of the row, H from the back), so the descriptor
// and force loops run species-uniform. Inference (k_mlp_bf16) runs the MLP
// forward and its backward to the input on the tensor cores with mma.sync
// m16n8k16 BF16 tiles (FP32 accumulate): one warp per 16 atoms of one
// species, weights staged once per block in shared memory (one orientation,
// ldmatrix / ldmatrix.trans give both), activations kept in registers in the
// A-fragment layout between layers. k_mlp_tc (NBG_MLP_TCGEN05) runs the same
// products with tcgen05.mma into tensor memory, 128 atoms per product. Learned forces are scattered to
// neighbours as 64-bit fixed point (2^-32 units) so the sum does not depend
// on the order of the atomics. Training runs in FP32 on the CUDA cores.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "nbg_internal.cuh"

#define ML_NK 24
#define ML_ND 64
#define ML_NH 128
#define ML_FQ 4294967296.0f  // fixed-point scale of the learned forces (2^32)

__constant__ float c_rho2inv[4];  // 1 / (2 rho_a^2)
__constant__ float c_alpha;       // Coulomb screening of the short-range target (1/nm)

struct MLView {
    // model (per species 0 = O, 1 = H)
    const float* theta[2];        // FP32 master parameters (layout of oracle/learned.py)
    const __nv_bfloat16* w1[2];   // W1 [64][128]
    const __nv_bfloat16* w2[2];   // W2 [128][128]
    // per atom
    const int* snbr;              // short list, column-major [k * n + i]
    const int* scount;            // nO | nH << 16
    int scap;
    float* x;                     // descriptor [n][64] (standardised, or raw)
    float* mom;                   // moments [n][2][4][9]: p (3) and Q (xx, yy, zz, xy, xz, yz)
    float* dx;                    // dE/dD [n][64]
    float* e;                     // E_i [n]
    unsigned long long* fq;       // learned force [3n], fixed point
    float rd2;                    // RD^2
    float rs2;                    // (RD + skin)^2 of the short list
};

static __device__ __forceinline__ int param_off_b1() { return ML_ND * ML_NH; }
static __device__ __forceinline__ int param_off_w2() { return ML_ND * ML_NH + ML_NH; }
static __device__ __forceinline__ int param_off_b2() { return ML_ND * ML_NH + ML_NH + ML_NH * ML_NH; }
static __device__ __forceinline__ int param_off_w3() { return param_off_b2() + ML_NH; }
static __device__ __forceinline__ int param_off_b3() { return param_off_w3() + ML_NH; }
static __device__ __forceinline__ int param_off_mu() { return param_off_b3() + 1; }
static __device__ __forceinline__ int param_off_sd() { return param_off_mu() + ML_ND; }
static __device__ __forceinline__ int param_off_muE() { return param_off_sd() + ML_ND; }

// fc = (cos(pi r / RD) + 1) / 2 and its derivative
__device__ __forceinline__ void ml_fc(float r, float& fc, float& dfc)
{
    float s, c;
    __sincosf(r * ((float)M_PI / ML_RD), &s, &c);
    fc = 0.5f * (c + 1.0f);
    dfc = -0.5f * ((float)M_PI / ML_RD) * s;
}

// g_k = scale * exp(-(t - k)^2 / 2) for k = 0..23 (t = (r - R0) / w) by a
// product recurrence from the middle centre k = 12: upwards
// g_{k+1} = g_k exp(t - k - 1/2), downwards g_{k-1} = g_k exp(k - t - 1/2),
// each ratio shrinking by 1/e per step. Both chains advance together in
// FP32x2: returns g_12 and gp[m] = (g_{13+m}, g_{11-m}), m = 0..11 (gp[11].x
// would be g_24 and is not a centre). Three exponentials instead of 24; for
// t > -1 every factor that matters stays a normal FP32 number (closer pairs,
// r < R0 - w, take the direct form).
__device__ __forceinline__ float ml_gauss_pairs(float t, float scale, float2* gp)
{
    const float d = t - 12.0f;
    if (d < -13.0f) {
#pragma unroll
        for (int m = 0; m < 12; ++m) {
            const float zu = t - (float)(13 + m), zd = t - (float)(11 - m);
            gp[m] = make_float2(scale * __expf(-0.5f * zu * zu), scale * __expf(-0.5f * zd * zd));
        }
        return scale * __expf(-0.5f * d * d);
    }
    const float g12 = scale * __expf(-0.5f * d * d);
    float2 cur = make_float2(g12, g12);
    float2 rat = make_float2(__expf(d - 0.5f), __expf(-d - 0.5f));
    const float2 einv = make_float2(0.36787944117144233f, 0.36787944117144233f);
#pragma unroll
    for (int m = 0; m < 12; ++m) {
        cur = __fmul2_rn(cur, rat);
        rat = __fmul2_rn(rat, einv);
        gp[m] = cur;
    }
    return g12;
}

// Candidates of one species column are gathered four at a time (indices,
// then split positions, all loads independent) and the pairs inside RD are
// staged per thread in shared memory, [slot][thread]; the arithmetic then
// runs over staged pairs only, so that lanes are not idled by rejected
// candidates and the gathers overlap.
#define ML_STAGE 24
#define ML_TPB 128

struct Stager {
    const int* col;
    int64_t n;
    int q, q1;
    // stage up to ML_STAGE pairs (r_j - r_i, j) into st[.][tid]; returns the count
    __device__ __forceinline__ int fill(const Dev& d, const RepDev& R, const float4& hi, const float4& lo, float rd2,
                                       float4 (*st)[ML_TPB], int tid)
    {
        int cnt = 0;
        while (q < q1 && cnt <= ML_STAGE - 4) {
            int jj[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) jj[u] = (q + u < q1) ? dbg_index(col[(int64_t)(q + u) * n], d.n, -1, d.status) : -1;
            float4 hh[4], ll[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                if (jj[u] >= 0) {
                    hh[u] = d.phi[jj[u]];
                    ll[u] = d.plo[jj[u]];
                }
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                if (jj[u] >= 0) {
                    const float3 dr = split_diff(hh[u], ll[u], hi, lo, true, R);  // r_j - r_i
                    const float r2 = dr.x * dr.x + dr.y * dr.y + dr.z * dr.z;
                    if (r2 < rd2) st[cnt++][tid] = make_float4(dr.x, dr.y, dr.z, __int_as_float(jj[u]));
                }
            }
            q += 4;
        }
        return cnt;
    }
};

// ---------------------------------------------------------------------
// short list: atoms of the long list within RD + skin, O neighbours from the
// front of the atom's column, H neighbours from the back (warp per atom;
// column-major so that thread-per-atom readers load a warp's entries in one
// transaction)
// ---------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_short_list(Dev d, MLView m, StepRef pos, int force, int* snbr, int* scount)
{
    const int parity = (int)(step_of(pos) & 1);
    const int lane = threadIdx.x % 32;
    const int64_t i = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / 32;
    if (i >= d.n) return;
    if (!(force || d.rebuild_flag[parity * d.nrep + d.rep_of[i]])) return;
    const RepDev& R = d.reps[d.rep_of[i]];
    const float4 hi = d.phi[i], lo = d.plo[i];
    const int cnt = d.nbr_count[i];
    const int* nl = d.nbr + i * d.nbr_istride;
    int* col = snbr + i;  // column-major: entry q at col[q * n]
    const unsigned below = (1u << lane) - 1u;
    int nO = 0, nH = 0;
    for (int k0 = 0; k0 < cnt; k0 += 32) {
        const int k = k0 + lane;
        bool take = false;
        int j = 0;
        if (k < cnt) {
            j = dbg_index(nl[(int64_t)k * d.nbr_kstride], d.n, (int)i, d.status);
            float3 dr = split_diff(hi, lo, d.phi[j], d.plo[j], true, R);
            take = dr.x * dr.x + dr.y * dr.y + dr.z * dr.z < m.rs2;
        }
        const bool isO = (j % 3) == 0;
        const unsigned bo = __ballot_sync(0xffffffffu, take && isO);
        const unsigned bh = __ballot_sync(0xffffffffu, take && !isO);
        if (take) {
            if (isO) {
                const int p = nO + __popc(bo & below);
                if (p < m.scap) col[(int64_t)p * d.n] = j;
            } else {
                const int p = nH + __popc(bh & below);
                if (p < m.scap) col[(int64_t)(m.scap - 1 - p) * d.n] = j;
            }
        }
        nO += __popc(bo);
        nH += __popc(bh);
    }
    if (lane == 0) {
        if (nO + nH > m.scap) {
            status_set(d.status, ST_SHORT_OVERFLOW);
            nO = min(nO, m.scap);
            nH = m.scap - nO;
        }
        scount[i] = nO | (nH << 16);
    }
}

// Walks entries q0..q1-1 of atom i's short-list column with the next
// neighbour's index and split position loaded one entry ahead, so that its
// gathers overlap the current pair's arithmetic.
struct NbrCursor {
    const int* col;
    int64_t stride;
    int q, q1;
    int jn;
    float4 hn, ln;
    __device__ __forceinline__ void load(const Dev& d)
    {
        if (q < q1) {
            jn = dbg_index(col[(int64_t)q * stride], d.n, 0, d.status);
            hn = d.phi[jn];
            ln = d.plo[jn];
        }
    }
    __device__ __forceinline__ NbrCursor(const Dev& d, const int* c, int64_t n, int a, int b)
        : col(c), stride(n), q(a), q1(b), jn(0)
    {
        load(d);
    }
    // current neighbour (index, split position) and advance
    __device__ __forceinline__ bool next(const Dev& d, int& j, float4& hj, float4& lj)
    {
        if (q >= q1) return false;
        j = jn;
        hj = hn;
        lj = ln;
        ++q;
        load(d);
        return true;
    }
};

// ---------------------------------------------------------------------
// descriptors (thread per atom). raw: write D unstandardised.
// ---------------------------------------------------------------------
__global__ void __launch_bounds__(ML_TPB) k_descriptor(Dev d, MLView m, int raw)
{
    __shared__ float4 st[ML_STAGE][ML_TPB];
    const int tid = threadIdx.x;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < d.n; i += (int64_t)gridDim.x * blockDim.x) {
        const RepDev& R = d.reps[d.rep_of[i]];
        const float4 hi = d.phi[i], lo = d.plo[i];
        const int cnt = m.scount[i];
        const float* th = (i % 3 == 0) ? m.theta[0] : m.theta[1];
        const float* mu = th + param_off_mu();
        const float* sd = th + param_off_sd();
        float* X = m.x + i * ML_ND;
        float* MO = m.mom + i * 72;
        for (int s = 0; s < 2; ++s) {
            Stager sg{m.snbr + i, d.n, s == 0 ? 0 : m.scap - (cnt >> 16), s == 0 ? (cnt & 0xffff) : m.scap};
            float G12 = 0.f;
            float2 G[12];
            float2 mo[4][5];  // p (x, y), (z, Qxx), (Qyy, Qzz), (Qxy, Qxz), (Qyz, -)
#pragma unroll
            for (int k = 0; k < 12; ++k) G[k] = make_float2(0.f, 0.f);
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int c = 0; c < 5; ++c) mo[a][c] = make_float2(0.f, 0.f);
            do {
                const int nst = sg.fill(d, R, hi, lo, m.rd2, st, tid);
                for (int c = 0; c < nst; ++c) {
                    const float4 e = st[c][tid];
                    const float r2 = e.x * e.x + e.y * e.y + e.z * e.z;
                    const float ir = rsqrtf(r2), r = r2 * ir;
                    const float ux = e.x * ir, uy = e.y * ir, uz = e.z * ir;
                    float f, df;
                    ml_fc(r, f, df);
                    float2 gp[12];
                    G12 += ml_gauss_pairs((r - ML_R0) * (1.0f / ML_W), f, gp);
#pragma unroll
                    for (int k = 0; k < 12; ++k) G[k] = __fadd2_rn(G[k], gp[k]);
                    const float2 comp[5] = {make_float2(ux, uy), make_float2(uz, ux * ux - (1.0f / 3.0f)),
                                            make_float2(uy * uy - (1.0f / 3.0f), uz * uz - (1.0f / 3.0f)),
                                            make_float2(ux * uy, ux * uz), make_float2(uy * uz, 0.f)};
#pragma unroll
                    for (int a = 0; a < 4; ++a) {
                        const float psi = f * __expf(-r2 * c_rho2inv[a]);
                        const float2 p2 = make_float2(psi, psi);
#pragma unroll
                        for (int c = 0; c < 5; ++c) mo[a][c] = __ffma2_rn(p2, comp[c], mo[a][c]);
                    }
                }
            } while (sg.q < sg.q1);
            // radial: G[k] for k = 13 + m (x) and 11 - m (y)
            float Gk[ML_NK];
            Gk[12] = G12;
#pragma unroll
            for (int k = 0; k < 12; ++k) {
                if (k < 11) Gk[13 + k] = G[k].x;
                Gk[11 - k] = G[k].y;
            }
#pragma unroll
            for (int k = 0; k < ML_NK; ++k) {
                const int col = s * ML_NK + k;
                X[col] = raw ? Gk[k] : (Gk[k] - mu[col]) / sd[col];
            }
#pragma unroll
            for (int a = 0; a < 4; ++a) {
                const float M[9] = {mo[a][0].x, mo[a][0].y, mo[a][1].x, mo[a][1].y, mo[a][2].x,
                                    mo[a][2].y, mo[a][3].x, mo[a][3].y, mo[a][4].x};
                const float A1 = M[0] * M[0] + M[1] * M[1] + M[2] * M[2];
                // |Q|_F^2 of the symmetric matrix (diagonal + 2 x off-diagonal)
                const float A2 = M[3] * M[3] + M[4] * M[4] + M[5] * M[5] + 2.f * (M[6] * M[6] + M[7] * M[7] + M[8] * M[8]);
                const int c1 = 48 + 4 * s + a, c2 = 56 + 4 * s + a;
                X[c1] = raw ? A1 : (A1 - mu[c1]) / sd[c1];
                X[c2] = raw ? A2 : (A2 - mu[c2]) / sd[c2];
#pragma unroll
                for (int c = 0; c < 9; ++c) MO[(s * 4 + a) * 9 + c] = M[c];
            }
        }
    }
}

// ---------------------------------------------------------------------
// MLP forward + backward to the input, BF16 tensor cores (mma.sync)
// ---------------------------------------------------------------------
__device__ __forceinline__ void mma_bf16(float* c, const unsigned* a, const unsigned* b)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ void ldsm_x4(unsigned* r, const void* p)
{
    const unsigned a = (unsigned)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(a));
}

__device__ __forceinline__ void ldsm_x4_t(unsigned* r, const void* p)
{
    const unsigned a = (unsigned)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(a));
}

__device__ __forceinline__ float tanh_fast(float x)
{
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ __forceinline__ unsigned pack_bf16(float lo, float hi)
{
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<unsigned*>(&v);
}

__device__ __forceinline__ unsigned pack_h2(float lo, float hi)
{
    __half2 v = __floats2half2_rn(lo, hi);
    return *reinterpret_cast<unsigned*>(&v);
}

__device__ __forceinline__ float2 unpack_h2(unsigned u)
{
    __half2 v = *reinterpret_cast<__half2*>(&u);
    return __half22float2(v);
}

#define MLP_WARPS 8
#define LDW (ML_NH + 8)  // bf16 row stride of the staged weights (272 B: ldmatrix rows spread over banks)
#define LDX (ML_ND + 8)  // bf16 row stride of a staged input tile (144 B)

struct MlpSmem {
    __nv_bfloat16 w1[ML_ND * LDW];  // W1 [input k][hidden n]
    __nv_bfloat16 w2[ML_NH * LDW];  // W2 [hidden k][hidden n]
    float b1[ML_NH], b2[ML_NH], w3[ML_NH], sdinv[ML_ND];
    __nv_bfloat16 xs[MLP_WARPS][16 * LDX];
    unsigned da1[MLP_WARPS][8 * 4 * 32];  // 1 - a1^2 as half2, in each lane's C-fragment order
};

// atom index of the k-th atom of a species in a water system (O = 3m; H = 3m+1, 3m+2)
__device__ __forceinline__ int64_t species_atom(int sp, int64_t k) { return sp == 0 ? 3 * k : 3 * (k / 2) + 1 + (k % 2); }

// Fragment layouts (m16n8k16, g = lane / 4, t = lane % 4): A a0..a3 = rows
// g, g+8 x columns 2t(+1), 2t+8(+1); B b0, b1 = rows 2t(+1), 2t+8(+1) x
// column g; C c0..c3 = rows g, g+8 x columns 2t(+1). The C tiles of output
// columns 16u..16u+15 are, packed to BF16, the A fragment of k-tile u of the
// next product, so activations never leave registers.
// Both species in one launch: blocks [0, blocks_o) take the O atoms, the
// rest the H atoms (each block stages one species' weights).
__global__ void __launch_bounds__(MLP_WARPS * 32, 2) k_mlp_bf16(MLView m, int64_t count_o, int64_t count_h,
                                                                 int blocks_o)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int sp = blockIdx.x < (unsigned)blocks_o ? 0 : 1;
    const int64_t count = sp == 0 ? count_o : count_h;
    const int64_t blk = sp == 0 ? blockIdx.x : blockIdx.x - blocks_o;
    const int64_t nblk = sp == 0 ? blocks_o : gridDim.x - blocks_o;
    MlpSmem& S = *reinterpret_cast<MlpSmem*>(smem_raw);
    const float* th = sp == 0 ? m.theta[0] : m.theta[1];
    {
        const uint4* g1 = reinterpret_cast<const uint4*>(sp == 0 ? m.w1[0] : m.w1[1]);
        const uint4* g2 = reinterpret_cast<const uint4*>(sp == 0 ? m.w2[0] : m.w2[1]);
        for (int e = threadIdx.x; e < ML_ND * 16; e += blockDim.x)
            reinterpret_cast<uint4*>(S.w1 + (e >> 4) * LDW)[e & 15] = g1[e];
        for (int e = threadIdx.x; e < ML_NH * 16; e += blockDim.x)
            reinterpret_cast<uint4*>(S.w2 + (e >> 4) * LDW)[e & 15] = g2[e];
        for (int e = threadIdx.x; e < ML_NH; e += blockDim.x) {
            S.b1[e] = th[param_off_b1() + e];
            S.b2[e] = th[param_off_b2() + e];
            S.w3[e] = th[param_off_w3() + e];
        }
        for (int e = threadIdx.x; e < ML_ND; e += blockDim.x) S.sdinv[e] = 1.0f / th[param_off_sd() + e];
    }
    __syncthreads();
    const float b3 = th[param_off_b3()];
    const float muE = th[param_off_muE()], sdE = th[param_off_muE() + 1];
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const int g = lane >> 2, t = lane & 3;
    __nv_bfloat16* xs = S.xs[warp];
    // per-lane ldmatrix row offsets
    const int rA = lane & 15, cA = (lane >> 4) * 8;                        // A (and trans-B) tiles
    const int rB = (lane >> 4) * 8 + (lane & 7), cB = ((lane >> 3) & 1) * 8;  // non-trans B tiles
    const int64_t ntile = (count + 15) / 16;
    for (int64_t tile = blk * MLP_WARPS + warp; tile < ntile; tile += nblk * MLP_WARPS) {
        const int64_t k0 = tile * 16;
        // 16 standardised descriptors to BF16 (rows past count are zero)
        for (int e = lane; e < 16 * 16; e += 32) {
            const int r = e >> 4, c4 = e & 15;
            const int64_t kk = k0 + r;
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (kk < count) v = reinterpret_cast<const float4*>(m.x + species_atom(sp, kk) * ML_ND)[c4];
            uint2 p;
            p.x = pack_bf16(v.x, v.y);
            p.y = pack_bf16(v.z, v.w);
            *reinterpret_cast<uint2*>(xs + r * LDX + 4 * c4) = p;
        }
        __syncwarp();
        unsigned xa[4][4];
#pragma unroll
        for (int kt = 0; kt < 4; ++kt) ldsm_x4(xa[kt], xs + rA * LDX + kt * 16 + cA);
        // layer 1: a1 = tanh(x W1 + b1), kept as A fragments; 1 - a1^2 as half2
        // in shared memory (each lane reads back only what it wrote)
        unsigned a1f[8][4];
        unsigned* d1h = S.da1[warp];
#pragma unroll
        for (int np = 0; np < 8; ++np) {
            float c0[4] = {0.f, 0.f, 0.f, 0.f}, c1[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int kt = 0; kt < 4; ++kt) {
                unsigned b[4];
                ldsm_x4_t(b, S.w1 + (kt * 16 + rA) * LDW + np * 16 + cA);
                mma_bf16(c0, xa[kt], b);
                mma_bf16(c1, xa[kt], b + 2);
            }
            const int col0 = np * 16 + 2 * t, col1 = col0 + 8;
            float v[8];
            v[0] = tanh_fast(c0[0] + S.b1[col0]);
            v[1] = tanh_fast(c0[1] + S.b1[col0 + 1]);
            v[2] = tanh_fast(c0[2] + S.b1[col0]);
            v[3] = tanh_fast(c0[3] + S.b1[col0 + 1]);
            v[4] = tanh_fast(c1[0] + S.b1[col1]);
            v[5] = tanh_fast(c1[1] + S.b1[col1 + 1]);
            v[6] = tanh_fast(c1[2] + S.b1[col1]);
            v[7] = tanh_fast(c1[3] + S.b1[col1 + 1]);
#pragma unroll
            for (int h = 0; h < 4; ++h) {
                a1f[np][h] = pack_bf16(v[2 * h], v[2 * h + 1]);
                d1h[(np * 4 + h) * 32 + lane] = pack_h2(1.f - v[2 * h] * v[2 * h], 1.f - v[2 * h + 1] * v[2 * h + 1]);
            }
        }
        // layer 2: a2 = tanh(a1 W2 + b2); E = sdE (a2.w3 + b3) + muE; g2 = sdE w3 (1 - a2^2)
        unsigned g2f[8][4];
        float er0 = 0.f, er1 = 0.f;
#pragma unroll
        for (int np = 0; np < 8; ++np) {
            float c0[4] = {0.f, 0.f, 0.f, 0.f}, c1[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int kt = 0; kt < 8; ++kt) {
                unsigned b[4];
                ldsm_x4_t(b, S.w2 + (kt * 16 + rA) * LDW + np * 16 + cA);
                mma_bf16(c0, a1f[kt], b);
                mma_bf16(c1, a1f[kt], b + 2);
            }
            const int col[2] = {np * 16 + 2 * t, np * 16 + 8 + 2 * t};
            const float* cc[2] = {c0, c1};
#pragma unroll
            for (int hh = 0; hh < 2; ++hh) {
                const int c = col[hh];
                const float w30 = S.w3[c], w31 = S.w3[c + 1];
                const float v0 = tanh_fast(cc[hh][0] + S.b2[c]), v1 = tanh_fast(cc[hh][1] + S.b2[c + 1]);
                const float v2 = tanh_fast(cc[hh][2] + S.b2[c]), v3 = tanh_fast(cc[hh][3] + S.b2[c + 1]);
                er0 += v0 * w30 + v1 * w31;
                er1 += v2 * w30 + v3 * w31;
                g2f[np][2 * hh] = pack_bf16(sdE * w30 * (1.f - v0 * v0), sdE * w31 * (1.f - v1 * v1));
                g2f[np][2 * hh + 1] = pack_bf16(sdE * w30 * (1.f - v2 * v2), sdE * w31 * (1.f - v3 * v3));
            }
        }
        // energies of rows g and g + 8 (sum over the quad)
        er0 += __shfl_xor_sync(0xffffffffu, er0, 1);
        er0 += __shfl_xor_sync(0xffffffffu, er0, 2);
        er1 += __shfl_xor_sync(0xffffffffu, er1, 1);
        er1 += __shfl_xor_sync(0xffffffffu, er1, 2);
        if (t == 0) {
            if (k0 + g < count) m.e[species_atom(sp, k0 + g)] = sdE * (er0 + b3) + muE;
            if (k0 + g + 8 < count) m.e[species_atom(sp, k0 + g + 8)] = sdE * (er1 + b3) + muE;
        }
        // backward 1: g1 = (g2 W2^T) (1 - a1^2); B(k, n) = W2[n][k]
        unsigned g1f[8][4];
#pragma unroll
        for (int np = 0; np < 8; ++np) {
            float c0[4] = {0.f, 0.f, 0.f, 0.f}, c1[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int kt = 0; kt < 8; ++kt) {
                unsigned b[4];
                ldsm_x4(b, S.w2 + (np * 16 + rB) * LDW + kt * 16 + cB);
                mma_bf16(c0, g2f[kt], b);
                mma_bf16(c1, g2f[kt], b + 2);
            }
            const float2 d0 = unpack_h2(d1h[(np * 4 + 0) * 32 + lane]), d1 = unpack_h2(d1h[(np * 4 + 1) * 32 + lane]);
            const float2 d2 = unpack_h2(d1h[(np * 4 + 2) * 32 + lane]), d3 = unpack_h2(d1h[(np * 4 + 3) * 32 + lane]);
            g1f[np][0] = pack_bf16(c0[0] * d0.x, c0[1] * d0.y);
            g1f[np][1] = pack_bf16(c0[2] * d1.x, c0[3] * d1.y);
            g1f[np][2] = pack_bf16(c1[0] * d2.x, c1[1] * d2.y);
            g1f[np][3] = pack_bf16(c1[2] * d3.x, c1[3] * d3.y);
        }
        // backward 2: dE/dD = (g1 W1^T) / sdD; B(k, n) = W1[n][k]
        const int64_t ag = k0 + g < count ? species_atom(sp, k0 + g) : -1;
        const int64_t ag8 = k0 + g + 8 < count ? species_atom(sp, k0 + g + 8) : -1;
#pragma unroll
        for (int np = 0; np < 4; ++np) {
            float c0[4] = {0.f, 0.f, 0.f, 0.f}, c1[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int kt = 0; kt < 8; ++kt) {
                unsigned b[4];
                ldsm_x4(b, S.w1 + (np * 16 + rB) * LDW + kt * 16 + cB);
                mma_bf16(c0, g1f[kt], b);
                mma_bf16(c1, g1f[kt], b + 2);
            }
            const int col0 = np * 16 + 2 * t, col1 = col0 + 8;
            if (ag >= 0) {
                float* D = m.dx + ag * ML_ND;
                *reinterpret_cast<float2*>(D + col0) = make_float2(c0[0] * S.sdinv[col0], c0[1] * S.sdinv[col0 + 1]);
                *reinterpret_cast<float2*>(D + col1) = make_float2(c1[0] * S.sdinv[col1], c1[1] * S.sdinv[col1 + 1]);
            }
            if (ag8 >= 0) {
                float* D = m.dx + ag8 * ML_ND;
                *reinterpret_cast<float2*>(D + col0) = make_float2(c0[2] * S.sdinv[col0], c0[3] * S.sdinv[col0 + 1]);
                *reinterpret_cast<float2*>(D + col1) = make_float2(c1[2] * S.sdinv[col1], c1[3] * S.sdinv[col1 + 1]);
            }
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------
// MLP forward + backward to the input on the fifth-generation tensor cores:
// tcgen05.mma from shared-memory operands into FP32 accumulators in tensor
// memory (TMEM), read back by tcgen05.ld for the epilogues.
// ---------------------------------------------------------------------
// A block is TC_GROUPS tile groups of 8 warps; each group takes 128-atom
// tiles of one species in turn. Per tile four products, each issued by one
// thread of the group and completing on the group's mbarrier:
//   D1 = X W1 (128 x 128, K 64)     a1 = tanh(D1 + b1)
//   D2 = a1 W2 (128 x 128, K 128)   a2 = tanh(D2 + b2), E, g2 = sdE w3 (1 - a2^2)
//   D3 = g2 W2^T                    g1 = D3 (1 - a1^2)
//   D4 = g1 W1^T (128 x 64)         dE/dD = D4 / sdD
// Warp w of a group reads TMEM lanes 32 (w % 4) .. + 31 (the lanes a warp
// may access) and the columns of half w / 4 of each product: a thread owns
// one tile row and half of its columns, so 1 - a1^2 stays in its registers
// (half2) from layer 1 to the first backward product, and the two halves of
// E meet in shared memory. The group's accumulator is 128 TMEM columns,
// reused by the four products.
//
// Operands use the K-major layout without swizzle: 8-row x 16-byte core
// matrices of 128 contiguous bytes; the core matrix of rows 8p.. and
// elements 8q.. of a tile with kd elements per row starts at
// p (16 kd) + 128 q bytes. In the shared-memory descriptor the first stride
// is the leading-dimension byte offset (128, between core matrices along K)
// and the second the stride byte offset (16 kd, between 8-row groups); one
// K step of 16 elements advances the start address by 256 bytes.
#define TC_GROUPS 2
#define TC_GT 256  // threads of a tile group
#define TC_WAIT_TRIES (1u << 24)

__device__ __forceinline__ unsigned ml_smem(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned tc_off(int r, int k, int kd)
{
    return (unsigned)((r >> 3) * (kd * 16) + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// shared-memory matrix descriptor: start >> 4 (bits 0-13), leading byte
// offset >> 4 (16-29), stride byte offset >> 4 (32-45), descriptor version 1
// (bits 46-47), base offset 0, no swizzle (bits 61-63 = 0)
__device__ __forceinline__ unsigned long long tc_sdesc(unsigned saddr, unsigned sbo)
{
    return (unsigned long long)((saddr & 0x3FFFFu) >> 4) | ((unsigned long long)(128u >> 4) << 16) |
           ((unsigned long long)(sbo >> 4) << 32) | (1ull << 46);
}

// kind::f16 instruction descriptor: FP32 accumulator (bits 4-5 = 1), BF16 A
// and B (bits 7-9, 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 at bit
// 17, M >> 4 at bit 24
__host__ __device__ constexpr unsigned tc_idesc(int M, int N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)(N >> 3) << 17) | ((unsigned)(M >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(unsigned dtm, unsigned long long ad, unsigned long long bd, unsigned idesc,
                                       unsigned acc)
{
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(dtm),
        "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void tc_commit(unsigned mbar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
                 : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ bool tc_mbar_try(unsigned a, unsigned parity)
{
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    return ok != 0;
}

// OR of a predicate over a tile group's threads at named barrier id
__device__ __forceinline__ bool tg_any(bool v, int id)
{
    unsigned r;
    asm volatile(
        "{\n .reg .pred q, p;\n setp.ne.u32 q, %1, 0;\n bar.red.or.pred p, %2, %3, q;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(r)
        : "r"((unsigned)v), "r"(id), "n"(TC_GT)
        : "memory");
    return r != 0;
}

__device__ __forceinline__ void tg_sync(int id) { asm volatile("bar.sync %0, %1;" ::"r"(id), "n"(TC_GT) : "memory"); }

#define TC_R8(a) "=r"(r[a]), "=r"(r[a + 1]), "=r"(r[a + 2]), "=r"(r[a + 3]), "=r"(r[a + 4]), "=r"(r[a + 5]), \
                 "=r"(r[a + 6]), "=r"(r[a + 7])
#define TC_W8(a) "+r"(r[a]), "+r"(r[a + 1]), "+r"(r[a + 2]), "+r"(r[a + 3]), "+r"(r[a + 4]), "+r"(r[a + 5]), \
                 "+r"(r[a + 6]), "+r"(r[a + 7])

// 32 consecutive FP32 columns of this thread's TMEM lane; the wait names the
// registers so that no use of them moves above it
__device__ __forceinline__ void tc_ld32(unsigned taddr, float (&v)[32])
{
    unsigned r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : TC_R8(0), TC_R8(8), TC_R8(16), TC_R8(24)
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" : TC_W8(0), TC_W8(8), TC_W8(16), TC_W8(24) : : "memory");
#pragma unroll
    for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(r[j]);
}

// thread gt's 8 float4 of the descriptors of the tile at species index k0
// (rows past count are zero)
__device__ __forceinline__ void tc_load_x(const MLView& m, int sp, int64_t count, int64_t k0, int gt, float4 (&xv)[8])
{
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int e = gt + TC_GT * i, r = e >> 4, c4 = e & 15;
        const int64_t kk = k0 + r;
        xv[i] = kk < count ? __ldg(reinterpret_cast<const float4*>(m.x + species_atom(sp, kk) * ML_ND) + c4)
                           : make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

struct TcSmem {
    __nv_bfloat16 w1t[ML_NH * ML_ND];          // B of X W1:     (n hidden, k input) = W1[k][n]
    __nv_bfloat16 w2t[ML_NH * ML_NH];          // B of a1 W2:    (n, k) = W2[k][n]
    __nv_bfloat16 w2[ML_NH * ML_NH];           // B of g2 W2^T:  (n, k) = W2[n][k]
    __nv_bfloat16 w1[ML_ND * ML_NH];           // B of g1 W1^T:  (n input, k hidden) = W1[n][k]
    __nv_bfloat16 xs[TC_GROUPS][128 * ML_ND];  // A: the tile's standardised descriptors
    __nv_bfloat16 hs[TC_GROUPS][128 * ML_NH];  // A: a1, then g2, then g1
    float b1[ML_NH], b2[ML_NH], w3[ML_NH], sw3[ML_NH], sdinv[ML_ND];  // sw3 = sdE w3
    float eh[TC_GROUPS][128];                  // the second column half's part of E
    unsigned long long mbar[TC_GROUPS];
    unsigned tmem;
};
static constexpr size_t TC_SMEM = sizeof(TcSmem) + 1024;  // + alignment of the operands to 1024 B

__global__ void __launch_bounds__(TC_GROUPS * TC_GT, 1) k_mlp_tc(MLView m, int64_t count_o, int64_t count_h,
                                                                 int blocks_o, unsigned* status)
{
    extern __shared__ __align__(16) unsigned char tc_raw[];
    TcSmem& S = *reinterpret_cast<TcSmem*>(tc_raw + ((1024u - (ml_smem(tc_raw) & 1023u)) & 1023u));
    const int sp = blockIdx.x < (unsigned)blocks_o ? 0 : 1;
    const int64_t count = sp == 0 ? count_o : count_h;
    const int64_t blk = sp == 0 ? blockIdx.x : blockIdx.x - blocks_o;
    const int64_t nblk = sp == 0 ? blocks_o : gridDim.x - blocks_o;
    const float* th = sp == 0 ? m.theta[0] : m.theta[1];  // (no dynamic index into the parameter)
    const int tid = threadIdx.x, grp = tid / TC_GT, gt = tid % TC_GT, warp = tid >> 5;
    const int row = (warp & 3) * 32 + (tid & 31);  // tile row = TMEM lane
    const int hf = (warp >> 2) & 1;                // column half of this warp
    {
        // W1 [64][128] and W2 [128][128] as 16-byte chunks of 8 columns, all
        // loads issued before the first store; a chunk of row k stays a row
        // of the straight tile and becomes 8 rows of the transposed one
        constexpr int NT = TC_GROUPS * TC_GT;
        constexpr int C1 = ML_ND * ML_NH / 8, C2 = ML_NH * ML_NH / 8, PER = (C1 + C2) / NT;
        static_assert((C1 + C2) % NT == 0 && C1 % NT == 0, "whole chunks per thread");
        const uint4* g1 = reinterpret_cast<const uint4*>(sp == 0 ? m.w1[0] : m.w1[1]);
        const uint4* g2 = reinterpret_cast<const uint4*>(sp == 0 ? m.w2[0] : m.w2[1]);
        uint4 ch[PER];
#pragma unroll
        for (int i = 0; i < PER; ++i) {
            const int c = tid + i * NT;
            ch[i] = c < C1 ? __ldg(g1 + c) : __ldg(g2 + (c - C1));
        }
#pragma unroll
        for (int i = 0; i < PER; ++i) {
            const int c0 = tid + i * NT;
            const bool one = c0 < C1;  // uniform over i
            const int c = one ? c0 : c0 - C1;
            const int k = c / 16, n0 = (c % 16) * 8;  // W[k][n0 .. n0 + 7]
            unsigned char* straight = reinterpret_cast<unsigned char*>(one ? S.w1 : S.w2);
            unsigned char* trans = reinterpret_cast<unsigned char*>(one ? S.w1t : S.w2t);
            const int kd = one ? ML_ND : ML_NH;  // K extent of the transposed tile
            *reinterpret_cast<uint4*>(straight + tc_off(k, n0, ML_NH)) = ch[i];
            const unsigned w4[4] = {ch[i].x, ch[i].y, ch[i].z, ch[i].w};
#pragma unroll
            for (int j = 0; j < 8; ++j)
                *reinterpret_cast<unsigned short*>(trans + tc_off(n0 + j, k, kd)) =
                    (unsigned short)(w4[j >> 1] >> (16 * (j & 1)));
        }
        for (int e = tid; e < ML_NH; e += blockDim.x) {
            S.b1[e] = th[param_off_b1() + e];
            S.b2[e] = th[param_off_b2() + e];
            S.w3[e] = th[param_off_w3() + e];
            S.sw3[e] = th[param_off_muE() + 1] * th[param_off_w3() + e];
        }
        for (int e = tid; e < ML_ND; e += blockDim.x) S.sdinv[e] = 1.0f / th[param_off_sd() + e];
    }
    if (tid < TC_GROUPS)
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(ml_smem(&S.mbar[tid])) : "memory");
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(ml_smem(&S.tmem)),
                     "r"(TC_GROUPS * 128)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    // the weights were written by generic stores and are read by the tensor cores
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const unsigned tcol = S.tmem + (unsigned)grp * 128u;               // this group's columns
    const unsigned trow = tcol + (((unsigned)(warp & 3) * 32u) << 16);  // this warp's 32 lanes
    const unsigned mb = ml_smem(&S.mbar[grp]);
    const int bar = 1 + grp;
    const unsigned sx = ml_smem(S.xs[grp]), sh = ml_smem(S.hs[grp]);
    const unsigned sw1t = ml_smem(S.w1t), sw2t = ml_smem(S.w2t), sw2 = ml_smem(S.w2), sw1 = ml_smem(S.w1);
    unsigned char* const xs = reinterpret_cast<unsigned char*>(S.xs[grp]);
    unsigned char* const hs = reinterpret_cast<unsigned char*>(S.hs[grp]);
    const float b3 = th[param_off_b3()];
    const float muE = th[param_off_muE()], sdE = th[param_off_muE() + 1];
    unsigned phase = 0;
    bool failed = false;
    // one product: operands written by this group's threads, then issued by
    // its thread 0 and completing on the group's mbarrier
    auto issue = [&](unsigned sa, unsigned sbo_a, unsigned sb, unsigned sbo_b, int ksteps, unsigned idesc) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        tc_fence_before();
        tg_sync(bar);
        if (gt == 0) {
            tc_fence_after();
            for (int s = 0; s < ksteps; ++s)
                tc_mma(tcol, tc_sdesc(sa + 256u * s, sbo_a), tc_sdesc(sb + 256u * s, sbo_b), idesc, s > 0);
            tc_commit(mb);
        }
    };
    // every thread waits (bounded) for the product; false if it did not
    // complete, decided the same way for the whole group
    auto done = [&]() {
        unsigned tries = 0;
        bool late = false;
        while (!tc_mbar_try(mb, phase)) {
            if (++tries > TC_WAIT_TRIES) {
                late = true;
                break;
            }
        }
        if (tg_any(late, bar)) return false;
        phase ^= 1u;
        tc_fence_after();
        return true;
    };
    // this thread's 8 float4 of a tile's descriptors (rows past count are zero)
    float4 xv[8];
    const int64_t ntile = (count + 127) / 128;
    const int64_t tstride = nblk * TC_GROUPS;
    if (blk * TC_GROUPS + grp < ntile) tc_load_x(m, sp, count, (blk * TC_GROUPS + grp) * 128, gt, xv);
    for (int64_t tile = blk * TC_GROUPS + grp; tile < ntile; tile += tstride) {
        const int64_t k0 = tile * 128;
        // the tile's descriptors to BF16
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int e = gt + TC_GT * i, r = e >> 4, c4 = e & 15;
            *reinterpret_cast<uint2*>(xs + tc_off(r, 4 * c4, ML_ND)) =
                make_uint2(pack_bf16(xv[i].x, xv[i].y), pack_bf16(xv[i].z, xv[i].w));
        }
        issue(sx, 16u * ML_ND, sw1t, 16u * ML_ND, ML_ND / 16, tc_idesc(128, ML_NH));
        if (!done()) {
            failed = true;
            break;
        }
        // layer 1 epilogue: a1 to the A tile, 1 - a1^2 kept as half2
        const float2 one2 = make_float2(1.f, 1.f);
        unsigned d1h[ML_NH / 4];
#pragma unroll
        for (int cc = 0; cc < 2; ++cc) {
            float v[32];
            const int c0 = hf * 64 + 32 * cc;
            tc_ld32(trow + (unsigned)c0, v);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                unsigned pk[4];
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int j = 8 * q + 4 * h;
                    const float4 bb = *reinterpret_cast<const float4*>(&S.b1[c0 + j]);
                    const float2 a01 = make_float2(tanh_fast(v[j] + bb.x), tanh_fast(v[j + 1] + bb.y));
                    const float2 a23 = make_float2(tanh_fast(v[j + 2] + bb.z), tanh_fast(v[j + 3] + bb.w));
                    pk[2 * h] = pack_bf16(a01.x, a01.y);
                    pk[2 * h + 1] = pack_bf16(a23.x, a23.y);
                    const float2 d01 = __ffma2_rn(make_float2(-a01.x, -a01.y), a01, one2);
                    const float2 d23 = __ffma2_rn(make_float2(-a23.x, -a23.y), a23, one2);
                    d1h[(32 * cc + j) / 2] = pack_h2(d01.x, d01.y);
                    d1h[(32 * cc + j) / 2 + 1] = pack_h2(d23.x, d23.y);
                }
                *reinterpret_cast<uint4*>(hs + tc_off(row, c0 + 8 * q, ML_NH)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
            }
        }
        issue(sh, 16u * ML_NH, sw2t, 16u * ML_NH, ML_NH / 16, tc_idesc(128, ML_NH));
        if (!done()) {
            failed = true;
            break;
        }
        // layer 2 epilogue: E (two halves), and g2 = sdE w3 (1 - a2^2) to the A tile
        float2 erp = make_float2(0.f, 0.f);
#pragma unroll
        for (int cc = 0; cc < 2; ++cc) {
            float v[32];
            const int c0 = hf * 64 + 32 * cc;
            tc_ld32(trow + (unsigned)c0, v);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                unsigned pk[4];
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int j = 8 * q + 4 * h, col = c0 + j;
                    const float4 bb = *reinterpret_cast<const float4*>(&S.b2[col]);
                    const float4 ww = *reinterpret_cast<const float4*>(&S.w3[col]);
                    const float4 sw = *reinterpret_cast<const float4*>(&S.sw3[col]);
                    const float2 a01 = make_float2(tanh_fast(v[j] + bb.x), tanh_fast(v[j + 1] + bb.y));
                    const float2 a23 = make_float2(tanh_fast(v[j + 2] + bb.z), tanh_fast(v[j + 3] + bb.w));
                    erp = __ffma2_rn(a01, make_float2(ww.x, ww.y), erp);
                    erp = __ffma2_rn(a23, make_float2(ww.z, ww.w), erp);
                    const float2 g01 = __fmul2_rn(make_float2(sw.x, sw.y),
                                                  __ffma2_rn(make_float2(-a01.x, -a01.y), a01, one2));
                    const float2 g23 = __fmul2_rn(make_float2(sw.z, sw.w),
                                                  __ffma2_rn(make_float2(-a23.x, -a23.y), a23, one2));
                    pk[2 * h] = pack_bf16(g01.x, g01.y);
                    pk[2 * h + 1] = pack_bf16(g23.x, g23.y);
                }
                *reinterpret_cast<uint4*>(hs + tc_off(row, c0 + 8 * q, ML_NH)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
            }
        }
        const float er = erp.x + erp.y;
        if (hf) S.eh[grp][row] = er;
        issue(sh, 16u * ML_NH, sw2, 16u * ML_NH, ML_NH / 16, tc_idesc(128, ML_NH));
        // (the group barrier in issue ordered the second half's part of E)
        const int64_t atom = k0 + row < count ? species_atom(sp, k0 + row) : -1;
        if (!hf && atom >= 0) m.e[atom] = sdE * ((er + S.eh[grp][row]) + b3) + muE;
        if (!done()) {
            failed = true;
            break;
        }
        // first backward epilogue: g1 = (g2 W2^T) (1 - a1^2) to the A tile
#pragma unroll
        for (int cc = 0; cc < 2; ++cc) {
            float v[32];
            const int c0 = hf * 64 + 32 * cc;
            tc_ld32(trow + (unsigned)c0, v);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                unsigned pk[4];
#pragma unroll
                for (int h = 0; h < 4; ++h) {
                    const int j = 8 * q + 2 * h;
                    const float2 g = __fmul2_rn(make_float2(v[j], v[j + 1]), unpack_h2(d1h[(32 * cc + j) / 2]));
                    pk[h] = pack_bf16(g.x, g.y);
                }
                *reinterpret_cast<uint4*>(hs + tc_off(row, c0 + 8 * q, ML_NH)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
            }
        }
        issue(sh, 16u * ML_NH, sw1, 16u * ML_NH, ML_NH / 16, tc_idesc(128, ML_ND));
        // the next tile's descriptors load while the last product runs
        if (tile + tstride < ntile) tc_load_x(m, sp, count, (tile + tstride) * 128, gt, xv);
        if (!done()) {
            failed = true;
            break;
        }
        // second backward epilogue: dE/dD = (g1 W1^T) / sdD, 32 columns per thread
        {
            float v[32];
            const int c0 = hf * 32;
            tc_ld32(trow + (unsigned)c0, v);
            if (atom >= 0) {
                float4* D = reinterpret_cast<float4*>(m.dx + atom * ML_ND + c0);
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const float4 sd = *reinterpret_cast<const float4*>(&S.sdinv[c0 + 4 * q]);
                    const float2 lo = __fmul2_rn(make_float2(v[4 * q], v[4 * q + 1]), make_float2(sd.x, sd.y));
                    const float2 hi = __fmul2_rn(make_float2(v[4 * q + 2], v[4 * q + 3]), make_float2(sd.z, sd.w));
                    D[q] = make_float4(lo.x, lo.y, hi.x, hi.y);
                }
            }
        }
    }
    if (failed) {
        if (gt == 0) status_set(status, ST_TIMEOUT);
        // the products still in flight write this block's TMEM: wait (bounded)
        unsigned tries = 0;
        while (!tc_mbar_try(mb, phase) && ++tries < TC_WAIT_TRIES) {
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(S.tmem), "r"(TC_GROUPS * 128)
                     : "memory");
    }
}

// ---------------------------------------------------------------------
// learned forces: F = -dE/dx through the descriptors (thread per atom i,
// scatter to the neighbours as fixed point)
// ---------------------------------------------------------------------
__device__ __forceinline__ void fq_add(unsigned long long* p, float v)
{
    atomicAdd(p, (unsigned long long)__float2ll_rn(v * ML_FQ));
}

__global__ void __launch_bounds__(ML_TPB) k_ml_force(Dev d, MLView m)
{
    __shared__ float4 st[ML_STAGE][ML_TPB];
    const int tid = threadIdx.x;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < d.n; i += (int64_t)gridDim.x * blockDim.x) {
        const RepDev& R = d.reps[d.rep_of[i]];
        const float4 hi = d.phi[i], lo = d.plo[i];
        const int cnt = m.scount[i];
        const float* dD = m.dx + i * ML_ND;  // dE/dD (already divided by sdD)
        const float* MO = m.mom + i * 72;
        float fi0 = 0.f, fi1 = 0.f, fi2 = 0.f;
        for (int s = 0; s < 2; ++s) {
            Stager sg{m.snbr + i, d.n, s == 0 ? 0 : m.scap - (cnt >> 16), s == 0 ? (cnt & 0xffff) : m.scap};
            if (sg.q >= sg.q1) continue;
            // coefficients in the pair order of ml_gauss_pairs: c_k and k c_k
            const float* cg = dD + s * ML_NK;
            const float c12 = cg[12];
            float2 cp[12], kp[12];
#pragma unroll
            for (int k = 0; k < 12; ++k) {
                const float cu = k < 11 ? cg[13 + k] : 0.f, cd = cg[11 - k];
                cp[k] = make_float2(cu, cd);
                kp[k] = make_float2((float)(13 + k) * cu, (float)(11 - k) * cd);
            }
            float cA1[4], cA2[4], P[4][3], Q[4][6];
#pragma unroll
            for (int a = 0; a < 4; ++a) {
                cA1[a] = 2.f * dD[48 + 4 * s + a];
                cA2[a] = 2.f * dD[56 + 4 * s + a];
#pragma unroll
                for (int c = 0; c < 3; ++c) P[a][c] = MO[(s * 4 + a) * 9 + c];
#pragma unroll
                for (int c = 0; c < 6; ++c) Q[a][c] = MO[(s * 4 + a) * 9 + 3 + c];
            }
            do {
                const int nst = sg.fill(d, R, hi, lo, m.rd2, st, tid);
                for (int c = 0; c < nst; ++c) {
                    const float4 e = st[c][tid];
                    const int j = __float_as_int(e.w);
                    const float r2 = e.x * e.x + e.y * e.y + e.z * e.z;
                    const float ir = rsqrtf(r2), r = r2 * ir;
                    const float ux = e.x * ir, uy = e.y * ir, uz = e.z * ir;
                    float f, df;
                    ml_fc(r, f, df);
                    const float tt = (r - ML_R0) * (1.0f / ML_W);
                    // radial: d(g_k fc)/dr = g_k (fc' - fc (t - k) / w); S0 = sum c_k g_k,
                    // S1 = sum c_k g_k (t - k) = t S0 - sum k c_k g_k
                    float2 gp[12];
                    const float g12 = ml_gauss_pairs(tt, 1.0f, gp);
                    float2 s0 = make_float2(c12 * g12, 0.f), sk = make_float2(12.f * c12 * g12, 0.f);
#pragma unroll
                    for (int k = 0; k < 12; ++k) {
                        s0 = __ffma2_rn(cp[k], gp[k], s0);
                        sk = __ffma2_rn(kp[k], gp[k], sk);
                    }
                    const float S0 = s0.x + s0.y;
                    const float S1 = tt * S0 - (sk.x + sk.y);
                    float sr = df * S0 - f * (1.0f / ML_W) * S1;  // coefficient of u
                    // angular: with psi_a, psi'_a and the moments p_a, Q_a,
                    // d|p|^2/dr_j = 2 [psi' (p.u) u + psi/r (p - (p.u) u)],
                    // d|Q|^2/dr_j = 2 [psi' (uQu) u + psi 2/r (Q u - (uQu) u)]
                    const float w6[6] = {ux * ux, uy * uy, uz * uz, 2.f * ux * uy, 2.f * ux * uz, 2.f * uy * uz};
                    float px = 0.f, py = 0.f, pz = 0.f;  // sum_a s2_a p_a
                    float W[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};  // sum_a t2_a Q_a
#pragma unroll
                    for (int a = 0; a < 4; ++a) {
                        const float ea = __expf(-r2 * c_rho2inv[a]);
                        const float psi = f * ea;
                        const float dpsi = ea * (df - 2.f * r * c_rho2inv[a] * f);
                        const float pu = P[a][0] * ux + P[a][1] * uy + P[a][2] * uz;
                        float uqu = 0.f;
#pragma unroll
                        for (int c = 0; c < 6; ++c) uqu = fmaf(Q[a][c], w6[c], uqu);
                        const float s2 = cA1[a] * psi * ir;
                        const float t2 = 2.f * cA2[a] * psi * ir;
                        sr += (cA1[a] * dpsi - s2) * pu + (cA2[a] * dpsi - t2) * uqu;
                        px = fmaf(s2, P[a][0], px);
                        py = fmaf(s2, P[a][1], py);
                        pz = fmaf(s2, P[a][2], pz);
#pragma unroll
                        for (int c = 0; c < 6; ++c) W[c] = fmaf(t2, Q[a][c], W[c]);
                    }
                    // W u with W = (xx, yy, zz, xy, xz, yz)
                    const float gx = sr * ux + px + W[0] * ux + W[3] * uy + W[4] * uz;
                    const float gy = sr * uy + py + W[3] * ux + W[1] * uy + W[5] * uz;
                    const float gz = sr * uz + pz + W[4] * ux + W[5] * uy + W[2] * uz;
                    fq_add(&m.fq[3 * j], -gx);
                    fq_add(&m.fq[3 * j + 1], -gy);
                    fq_add(&m.fq[3 * j + 2], -gz);
                    fi0 += gx;
                    fi1 += gy;
                    fi2 += gz;
                }
            } while (sg.q < sg.q1);
        }
        fq_add(&m.fq[3 * i], fi0);
        fq_add(&m.fq[3 * i + 1], fi1);
        fq_add(&m.fq[3 * i + 2], fi2);
    }
}

// ---------------------------------------------------------------------
// exact short-range energies and forces (labels and judge), thread per atom
// ---------------------------------------------------------------------
__device__ __forceinline__ void smoothstep(float r, float& S, float& dS)
{
    float t = (r - ML_RS) * (1.0f / (ML_RD - ML_RS));
    t = fminf(1.f, fmaxf(0.f, t));
    const float t2 = t * t, t3 = t2 * t;
    S = 1.f - 10.f * t3 + 15.f * t3 * t - 6.f * t3 * t2;
    dS = (-30.f * t2 + 60.f * t3 - 30.f * t3 * t) * (1.0f / (ML_RD - ML_RS));
}

__global__ void __launch_bounds__(ML_TPB) k_sr_exact(Dev d, MLView m, float* e_out, float* f_out, double* a_out)
{
    const float eps4 = (float)(4.0 * d.lj_eps);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < d.n; i += (int64_t)gridDim.x * blockDim.x) {
        const RepDev& R = d.reps[d.rep_of[i]];
        const float4 hi = d.phi[i], lo = d.plo[i];
        const int cnt = m.scount[i];
        const float kqi = (float)(d.el_k_d * d.charge[i]);
        const bool oi = (i % 3 == 0);
        float E = 0.f, fx = 0.f, fy = 0.f, fz = 0.f;
        for (int s = 0; s < 2; ++s) {
            const int q0 = s == 0 ? 0 : m.scap - (cnt >> 16);
            const int q1 = s == 0 ? (cnt & 0xffff) : m.scap;
            const bool lj_pair = oi && s == 0;  // LJ acts between O atoms only
            NbrCursor cur(d, m.snbr + i, d.n, q0, q1);
            int j;
            float4 hj, lj;
            while (cur.next(d, j, hj, lj)) {
                const float3 dr = split_diff(hj, lj, hi, lo, true, R);  // r_j - r_i
                const float r2 = dr.x * dr.x + dr.y * dr.y + dr.z * dr.z;
                if (!(r2 < m.rd2)) continue;
                const float ir = rsqrtf(r2), r = r2 * ir;
                // screened Coulomb k q q erfc(a r) / r and its r-derivative
                const float kqq = kqi * (float)d.charge[j];
                const float ec = erfcf(c_alpha * r);
                float phi = kqq * ec * ir;
                float dphi = -phi * ir - kqq * ir * (1.1283791670955126f * c_alpha) * __expf(-c_alpha * c_alpha * r2);
                if (lj_pair) {
                    const float s2 = d.lj_sig2 * ir * ir, s6 = s2 * s2 * s2;
                    phi += eps4 * (s6 * s6 - s6);
                    dphi += eps4 * (-12.f * s6 * s6 + 6.f * s6) * ir;
                }
                float S, dS;
                smoothstep(r, S, dS);
                E += 0.5f * phi * S;
                // F_i = d(phi S)/dr (r_j - r_i) / r for the pair energy phi S
                const float fp = (dphi * S + phi * dS) * ir;
                fx += fp * dr.x;
                fy += fp * dr.y;
                fz += fp * dr.z;
            }
        }
        if (e_out) e_out[i] = E;
        if (f_out) {
            f_out[3 * i] = fx;
            f_out[3 * i + 1] = fy;
            f_out[3 * i + 2] = fz;
        }
        if (a_out) {
            const double im = d.inv_mass[i];
            a_out[3 * i] = (double)fx * im;
            a_out[3 * i + 1] = (double)fy * im;
            a_out[3 * i + 2] = (double)fz * im;
        }
    }
}

// ---------------------------------------------------------------------
// training (FP32, CUDA cores)
// ---------------------------------------------------------------------
// Forward and backward of one batch: thread per sample b. X rows are raw
// descriptors (standardised here; std != 0 uses them already standardised),
// y raw labels. Writes x, a1, a2, g1, g2 ([B][128]) and e ([B]: dL/dout);
// loss into *loss (atomic, FP64).
__global__ void __launch_bounds__(64) k_train_fb(const float* __restrict__ theta, const float* __restrict__ X,
                                                 const float* __restrict__ Y, const int* __restrict__ idx, int B,
                                                 int standardised, float* xs, float* a1, float* a2, float* g1,
                                                 float* g2, float* eo, double* loss)
{
    extern __shared__ float sw[];
    float* W1 = sw;                  // [64][128]
    float* W2 = W1 + ML_ND * ML_NH;  // [128][128]
    for (int e = threadIdx.x; e < ML_ND * ML_NH; e += blockDim.x) W1[e] = theta[e];
    for (int e = threadIdx.x; e < ML_NH * ML_NH; e += blockDim.x) W2[e] = theta[param_off_w2() + e];
    __syncthreads();
    const float* b1 = theta + param_off_b1();
    const float* b2 = theta + param_off_b2();
    const float* w3 = theta + param_off_w3();
    const float b3 = theta[param_off_b3()];
    const float* mu = theta + param_off_mu();
    const float* sd = theta + param_off_sd();
    const float muE = theta[param_off_muE()], sdE = theta[param_off_muE() + 1];
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    const int row = idx ? idx[b] : b;
    const float* D = X + (int64_t)row * ML_ND;
    float* xb = xs + (int64_t)b * ML_ND;
    for (int k = 0; k < ML_ND; ++k) xb[k] = standardised ? D[k] : (D[k] - mu[k]) / sd[k];
    float* A1 = a1 + (int64_t)b * ML_NH;
    float* A2 = a2 + (int64_t)b * ML_NH;
    for (int n = 0; n < ML_NH; ++n) {
        float z = b1[n];
        for (int k = 0; k < ML_ND; ++k) z = fmaf(xb[k], W1[k * ML_NH + n], z);
        A1[n] = tanhf(z);
    }
    float out = b3;
    for (int n = 0; n < ML_NH; ++n) {
        float z = b2[n];
        for (int k = 0; k < ML_NH; ++k) z = fmaf(A1[k], W2[k * ML_NH + n], z);
        const float v = tanhf(z);
        A2[n] = v;
        out = fmaf(v, w3[n], out);
    }
    const float y = standardised ? Y[row] : (Y[row] - muE) / sdE;
    const float err = out - y;
    atomicAdd(loss, (double)err * (double)err / (double)B);
    const float de = 2.f * err / (float)B;
    eo[b] = de;
    float* G2 = g2 + (int64_t)b * ML_NH;
    float* G1 = g1 + (int64_t)b * ML_NH;
    for (int n = 0; n < ML_NH; ++n) G2[n] = de * w3[n] * (1.f - A2[n] * A2[n]);
    for (int k = 0; k < ML_NH; ++k) {
        float s = 0.f;
        for (int n = 0; n < ML_NH; ++n) s = fmaf(G2[n], W2[k * ML_NH + n], s);
        G1[k] = s * (1.f - A1[k] * A1[k]);
    }
}

// grad[p] for W1 (64x128), b1, W2 (128x128), b2, w3, b3: column sums over the
// batch in fixed order (thread per parameter)
__global__ void k_train_grad(int B, const float* __restrict__ xs, const float* __restrict__ a1,
                             const float* __restrict__ a2, const float* __restrict__ g1, const float* __restrict__ g2,
                             const float* __restrict__ eo, float* grad)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const int nW1 = ML_ND * ML_NH, nW2 = ML_NH * ML_NH;
    if (p >= ML_NTRAIN) return;
    float s = 0.f;
    if (p < nW1) {
        const int k = p / ML_NH, n = p % ML_NH;
        for (int b = 0; b < B; ++b) s = fmaf(xs[(int64_t)b * ML_ND + k], g1[(int64_t)b * ML_NH + n], s);
    } else if (p < nW1 + ML_NH) {
        const int n = p - nW1;
        for (int b = 0; b < B; ++b) s += g1[(int64_t)b * ML_NH + n];
    } else if (p < nW1 + ML_NH + nW2) {
        const int q = p - nW1 - ML_NH, k = q / ML_NH, n = q % ML_NH;
        for (int b = 0; b < B; ++b) s = fmaf(a1[(int64_t)b * ML_NH + k], g2[(int64_t)b * ML_NH + n], s);
    } else if (p < nW1 + 2 * ML_NH + nW2) {
        const int n = p - nW1 - ML_NH - nW2;
        for (int b = 0; b < B; ++b) s += g2[(int64_t)b * ML_NH + n];
    } else if (p < nW1 + 3 * ML_NH + nW2) {
        const int n = p - nW1 - 2 * ML_NH - nW2;
        for (int b = 0; b < B; ++b) s = fmaf(a2[(int64_t)b * ML_NH + n], eo[b], s);
    } else {
        for (int b = 0; b < B; ++b) s += eo[b];
    }
    grad[p] = s;
}

// Adam (Kingma & Ba 2015) on the trainable parameters
__global__ void k_adam(float* theta, const float* grad, float* m1, float* m2, int count, float lr, float b1, float b2,
                       float eps, float c1, float c2)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= count) return;
    const float g = grad[p];
    const float a = b1 * m1[p] + (1.f - b1) * g;
    const float v = b2 * m2[p] + (1.f - b2) * g * g;
    m1[p] = a;
    m2[p] = v;
    theta[p] -= lr * (a / c1) / (sqrtf(v / c2) + eps);
}

// BF16 copies of W1 and W2 for inference
__global__ void k_ml_pack_bf16(const float* theta, __nv_bfloat16* w1, __nv_bfloat16* w2)
{
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ML_NH * ML_NH; e += gridDim.x * blockDim.x) {
        if (e < ML_ND * ML_NH) w1[e] = __float2bfloat16_rn(theta[e]);
        w2[e] = __float2bfloat16_rn(theta[param_off_w2() + e]);
    }
}

// copy one species' rows of the raw descriptors and labels into the training set
__global__ void k_ml_collect(const float* x, const float* e, int64_t n, int sp, float* X, float* Y, int64_t off,
                             int64_t cap)
{
    const int64_t per = sp == 0 ? n / 3 : 2 * (n / 3);
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < per; k += (int64_t)gridDim.x * blockDim.x) {
        if (off + k >= cap) return;
        const int64_t i = species_atom(sp, k);
        for (int c = 0; c < ML_ND; ++c) X[(off + k) * ML_ND + c] = x[i * ML_ND + c];
        Y[off + k] = e[i];
    }
}

// mean and standard deviation of each descriptor column and of the labels
// (one block per column, FP64 sums in fixed order)
__global__ void k_ml_stats(const float* X, const float* Y, int64_t rows, float* theta)
{
    const int col = blockIdx.x;  // 0..63 descriptors, 64 = labels
    double s = 0.0, s2 = 0.0;
    for (int64_t r = threadIdx.x; r < rows; r += blockDim.x) {
        const double v = col < ML_ND ? X[r * ML_ND + col] : Y[r];
        s += v;
        s2 += v * v;
    }
    __shared__ double a[256], b[256];
    a[threadIdx.x] = s;
    b[threadIdx.x] = s2;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            a[threadIdx.x] += a[threadIdx.x + w];
            b[threadIdx.x] += b[threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double mean = a[0] / (double)rows;
        const double var = b[0] / (double)rows - mean * mean;
        const double sd = sqrt(var > 1e-12 ? var : 1e-12);
        if (col < ML_ND) {
            theta[param_off_mu() + col] = (float)mean;
            theta[param_off_sd() + col] = (float)sd;
        } else {
            theta[param_off_muE()] = (float)mean;
            theta[param_off_muE() + 1] = (float)sd;
        }
    }
}

// random sample indices for a batch (Philox, seed and batch counter)
__global__ void k_ml_sample(int* idx, int B, int64_t rows, uint64_t seed, uint64_t batch)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    const uint4 w = philox(seed, (uint64_t)b, batch, 7u);
    const uint64_t r = ((uint64_t)w.x << 32) | w.y;
    idx[b] = (int)(r % (uint64_t)rows);
}

// a (=, +=, -=) F / m from the fixed-point learned forces (mode 0, 1, -1)
__global__ void k_ml_accel(const unsigned long long* fq, const double* mass, int64_t n, int mode, double* a)
{
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < 3 * n; e += (int64_t)gridDim.x * blockDim.x) {
        const double f = (double)(long long)fq[e] * (1.0 / 4294967296.0);
        const double v = f / mass[e / 3];
        a[e] = mode == 0 ? v : (mode > 0 ? a[e] + v : a[e] - v);
    }
}

// learned forces as FP64 (host export)
__global__ void k_ml_force_out(const unsigned long long* fq, int64_t n, double* f)
{
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < 3 * n; e += (int64_t)gridDim.x * blockDim.x)
        f[e] = (double)(long long)fq[e] * (1.0 / 4294967296.0);
}

// judge sums: |F_ml - F_sr|^2 and |F_sr|^2 into acc[slot][0..1]
__global__ void k_ml_judge(const unsigned long long* fq, const float* fsr, int64_t n, double* acc, StepRef sr,
                           int inner, int slots)
{
    double s1 = 0.0, s2 = 0.0;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < 3 * n; e += (int64_t)gridDim.x * blockDim.x) {
        const double fm = (double)(long long)fq[e] * (1.0 / 4294967296.0);
        const double dlt = fm - (double)fsr[e];
        s1 += dlt * dlt;
        s2 += (double)fsr[e] * (double)fsr[e];
    }
    for (int o = 16; o > 0; o >>= 1) {
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
        s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    }
    const int64_t slot = ((step_of(sr) / inner) % slots + slots) % slots;
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(acc + 2 * slot, s1);
        atomicAdd(acc + 2 * slot + 1, s2);
    }
}

// outer r-RESPA kick: v += h (a_slow + Berendsen term at T of v), T read
// from red_T (the temperature of v, reduced by the kick that produced v).
// With Berendsen it also reduces sum m v'^2 of its output into red_T (block
// partials; the last block to finish adds them in block order).
__global__ void __launch_bounds__(256) k_respa_kick(Dev d, double* v, const double* a, double h, double* part,
                                                    unsigned* counter)
{
    const bool berendsen = d.therm == NBG_THERMO_BERENDSEN;
    // the Berendsen factor once per block (its FP64 divisions are long
    // sequences on this GPU's FP64 pipe)
    double fac = 0.0;
    if (berendsen) {
        __shared__ double fac_s;
        if (threadIdx.x == 0) {
            const double T = d.red_T[0];
            const RepDev& R = d.reps[0];
            const double gm = 0.5 / R.tparam;
            fac_s = (1.0 / T == INFINITY) ? gm : gm * (R.T0 / T - 1.0);
        }
        __syncthreads();
        fac = fac_s;
    }
    double acc = 0.0;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < 3 * d.n; e += (int64_t)gridDim.x * blockDim.x) {
        double an = a[e];
        if (berendsen) an += fac * v[e];
        if (!isfinite(an)) status_set(d.status, ST_NONFINITE);
        const double vn = v[e] + h * an;
        v[e] = vn;
        if (berendsen) acc += d.mass[e / 3] * (vn * vn);
    }
    if (!berendsen) return;
    __shared__ double sh[256];
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    __shared__ bool last;
    if (threadIdx.x == 0) {
        part[blockIdx.x] = sh[0];
        __threadfence();
        last = (atomicAdd(counter, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double t = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) t += ((volatile double*)part)[b];
    sh[threadIdx.x] = t;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        d.red_T[0] = sh[0] / (d.kb * d.reps[0].ndf);
        *counter = 0u;
    }
}

// ---------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------
int ml_init_constants()
{
    const float rho[4] = {ML_RHO0, ML_RHO1, ML_RHO2, ML_RHO3};
    float v[4];
    for (int a = 0; a < 4; ++a) v[a] = 1.0f / (2.0f * rho[a] * rho[a]);
    if (cudaMemcpyToSymbol(c_rho2inv, v, sizeof(v)) != cudaSuccess) return NBG_ERR_CUDA;
    const float alpha = ML_ALPHA;
    return cudaMemcpyToSymbol(c_alpha, &alpha, sizeof(alpha)) == cudaSuccess ? NBG_OK : NBG_ERR_CUDA;
}

size_t ml_mlp_smem() { return sizeof(MlpSmem); }

static MLView ml_view(nbg_ctx* c)
{
    MLView m;
    for (int s = 0; s < 2; ++s) {
        m.theta[s] = c->ml_theta[s];
        m.w1[s] = c->ml_w1[s];
        m.w2[s] = c->ml_w2[s];
    }
    m.snbr = c->ml_snbr;
    m.scount = c->ml_scnt;
    m.scap = c->ml_scap;
    m.x = c->ml_x;
    m.mom = c->ml_mom;
    m.dx = c->ml_dx;
    m.e = c->ml_e;
    m.fq = c->ml_fq;
    m.rd2 = ML_RD * ML_RD;
    const float rs = ML_RD + (float)c->desc.skin;
    m.rs2 = rs * rs * (1.0f + 1e-5f);
    return m;
}

int launch_short_list(nbg_ctx* c, StepRef pos, bool force)
{
    MLView m = ml_view(c);
    k_short_list<<<grid_for(c->n * 32, 256), 256, 0, c->stream>>>(c->d, m, pos, force ? 1 : 0, c->ml_snbr, c->ml_scnt);
    NBG_LAUNCH_CHECK(c, "k_short_list");
    return NBG_OK;
}

int launch_descriptor(nbg_ctx* c, bool raw)
{
    k_descriptor<<<grid_for(c->n, ML_TPB), ML_TPB, 0, c->stream>>>(c->d, ml_view(c), raw ? 1 : 0);
    NBG_LAUNCH_CHECK(c, "k_descriptor");
    return NBG_OK;
}

// blocks of one launch over both species, split by their tiles: all of
// them when they fit in `slots` resident blocks, else `slots` in proportion
static void mlp_split(int64_t tiles_o, int64_t tiles_h, int64_t per_block, int64_t slots, int64_t& bo, int64_t& bh)
{
    bo = (tiles_o + per_block - 1) / per_block;
    bh = (tiles_h + per_block - 1) / per_block;
    if (bo + bh > slots) {
        bo = std::max<int64_t>(1, (slots * tiles_o + (tiles_o + tiles_h) / 2) / (tiles_o + tiles_h));
        bh = std::max<int64_t>(1, slots - bo);
    }
}

int launch_mlp(nbg_ctx* c)
{
    if (!c->ml_attr) {
        int st = launch_mlp_attrs(c);
        if (st) return st;
    }
    const MLView m = ml_view(c);
    const int64_t count_o = c->n / 3, count_h = 2 * (c->n / 3);
    int64_t bo, bh;
    if (getenv("NBG_MLP_TCGEN05")) {
        // the tensor-memory form: one block per SM (its shared memory),
        // 128-atom tiles per group of 8 warps
        mlp_split((count_o + 127) / 128, (count_h + 127) / 128, TC_GROUPS, (int64_t)c->sms, bo, bh);
        k_mlp_tc<<<(int)(bo + bh), TC_GROUPS * TC_GT, TC_SMEM, c->stream>>>(m, count_o, count_h, (int)bo,
                                                                             c->d.status);
        NBG_LAUNCH_CHECK(c, "k_mlp_tc");
        return NBG_OK;
    }
    // the warp-level form (the faster at these layer sizes): two resident
    // blocks per SM, 16-atom tiles per warp
    mlp_split((count_o + 15) / 16, (count_h + 15) / 16, MLP_WARPS, (int64_t)c->sms * 2, bo, bh);
    k_mlp_bf16<<<(int)(bo + bh), MLP_WARPS * 32, sizeof(MlpSmem), c->stream>>>(m, count_o, count_h, (int)bo);
    NBG_LAUNCH_CHECK(c, "k_mlp_bf16");
    return NBG_OK;
}

int launch_ml_force(nbg_ctx* c)
{
    cudaError_t e = cudaMemsetAsync(c->ml_fq, 0, sizeof(unsigned long long) * 3 * c->n, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "ml force clear");
    k_ml_force<<<grid_for(c->n, ML_TPB), ML_TPB, 0, c->stream>>>(c->d, ml_view(c));
    NBG_LAUNCH_CHECK(c, "k_ml_force");
    return NBG_OK;
}

int launch_sr_exact(nbg_ctx* c, float* e_out, float* f_out, double* a_out)
{
    k_sr_exact<<<grid_for(c->n, 128), 128, 0, c->stream>>>(c->d, ml_view(c), e_out, f_out, a_out);
    NBG_LAUNCH_CHECK(c, "k_sr_exact");
    return NBG_OK;
}

int launch_ml_accel(nbg_ctx* c, int mode, double* a)
{
    k_ml_accel<<<grid_for(3 * c->n, 256), 256, 0, c->stream>>>(c->ml_fq, c->d.mass, c->n, mode, a);
    NBG_LAUNCH_CHECK(c, "k_ml_accel");
    return NBG_OK;
}

int launch_sr_inner(nbg_ctx* c, StepRef pos, bool force_short, double* a_out)
{
    int st;
    if ((st = launch_short_list(c, pos, force_short))) return st;
    return launch_sr_exact(c, nullptr, c->ml_fsr, a_out);
}

// a (=, +=, -=) F / m from FP32 forces (the exact short-range force)
__global__ void k_accel_from_f32(const float* f, const double* inv_mass, int64_t n, int mode, double* a)
{
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < 3 * n; e += (int64_t)gridDim.x * blockDim.x) {
        const double v = (double)f[e] * inv_mass[e / 3];
        a[e] = mode == 0 ? v : (mode > 0 ? a[e] + v : a[e] - v);
    }
}

int launch_sr_accel(nbg_ctx* c, int mode, double* a)
{
    k_accel_from_f32<<<grid_for(3 * c->n, 256), 256, 0, c->stream>>>(c->ml_fsr, c->d.inv_mass, c->n, mode, a);
    NBG_LAUNCH_CHECK(c, "k_accel_from_f32");
    return NBG_OK;
}

int launch_ml_force_out(nbg_ctx* c, double* f)
{
    k_ml_force_out<<<grid_for(3 * c->n, 256), 256, 0, c->stream>>>(c->ml_fq, c->n, f);
    NBG_LAUNCH_CHECK(c, "k_ml_force_out");
    return NBG_OK;
}

int launch_ml_judge(nbg_ctx* c, StepRef sr, int inner, int slots)
{
    k_ml_judge<<<std::min(grid_for(3 * c->n, 256), 1024), 256, 0, c->stream>>>(c->ml_fq, c->ml_fsr, c->n, c->ml_judge,
                                                                                   sr, inner, slots);
    NBG_LAUNCH_CHECK(c, "k_ml_judge");
    return NBG_OK;
}

int launch_respa_kick(nbg_ctx* c, double* v, const double* a, double h)
{
    const int grid = std::min(grid_for(3 * c->n, 256), c->kick_blocks);
    k_respa_kick<<<grid, 256, 0, c->stream>>>(c->d, v, a, h, c->kick_part, c->kick_counter);
    NBG_LAUNCH_CHECK(c, "k_respa_kick");
    return NBG_OK;
}

int launch_ml_pack(nbg_ctx* c, int sp)
{
    k_ml_pack_bf16<<<64, 256, 0, c->stream>>>(c->ml_theta[sp], c->ml_w1[sp], c->ml_w2[sp]);
    NBG_LAUNCH_CHECK(c, "k_ml_pack_bf16");
    return NBG_OK;
}

int launch_ml_collect(nbg_ctx* c, int sp, int64_t off)
{
    k_ml_collect<<<grid_for(c->n, 128), 128, 0, c->stream>>>(c->ml_x, c->ml_esr, c->n, sp, c->ml_X[sp], c->ml_Y[sp],
                                                            off, c->ml_cap[sp]);
    NBG_LAUNCH_CHECK(c, "k_ml_collect");
    return NBG_OK;
}

int launch_ml_stats(nbg_ctx* c, int sp)
{
    k_ml_stats<<<ML_ND + 1, 256, 0, c->stream>>>(c->ml_X[sp], c->ml_Y[sp], c->ml_rows[sp], c->ml_theta[sp]);
    NBG_LAUNCH_CHECK(c, "k_ml_stats");
    return NBG_OK;
}

static int train_fb_grad(nbg_ctx* c, const float* theta, const float* X, const float* Y, const int* idx, int B,
                         bool standardised, MLTrainScratch& s)
{
    const int smem = (ML_ND * ML_NH + ML_NH * ML_NH) * (int)sizeof(float);
    k_train_fb<<<(B + 63) / 64, 64, smem, c->stream>>>(theta, X, Y, idx, B, standardised ? 1 : 0, s.xs, s.a1, s.a2,
                                                       s.g1, s.g2, s.eo, s.loss);
    NBG_LAUNCH_CHECK(c, "k_train_fb");
    k_train_grad<<<(ML_NTRAIN + 127) / 128, 128, 0, c->stream>>>(B, s.xs, s.a1, s.a2, s.g1, s.g2, s.eo, s.grad);
    NBG_LAUNCH_CHECK(c, "k_train_grad");
    return NBG_OK;
}

int launch_ml_train_step(nbg_ctx* c, int sp, int B, uint64_t seed, uint64_t batch, float lr, int64_t t_adam)
{
    MLTrainScratch& s = c->ml_ts;
    if (!c->ml_attr) {
        int st = launch_mlp_attrs(c);
        if (st) return st;
    }
    k_ml_sample<<<(B + 255) / 256, 256, 0, c->stream>>>(s.idx, B, c->ml_rows[sp], seed, batch);
    NBG_LAUNCH_CHECK(c, "k_ml_sample");
    int st = train_fb_grad(c, c->ml_theta[sp], c->ml_X[sp], c->ml_Y[sp], s.idx, B, false, s);
    if (st) return st;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - powf(b1, (float)t_adam), c2 = 1.f - powf(b2, (float)t_adam);
    k_adam<<<(ML_NTRAIN + 255) / 256, 256, 0, c->stream>>>(c->ml_theta[sp], s.grad, s.m1[sp], s.m2[sp], ML_NTRAIN, lr,
                                                           b1, b2, 1e-8f, c1, c2);
    NBG_LAUNCH_CHECK(c, "k_adam");
    return NBG_OK;
}

int launch_ml_batch_grad(nbg_ctx* c, const float* theta, const float* X, const float* Y, int B)
{
    if (!c->ml_attr) {
        int st = launch_mlp_attrs(c);
        if (st) return st;
    }
    return train_fb_grad(c, theta, X, Y, nullptr, B, true, c->ml_ts);
}

int launch_mlp_attrs(nbg_ctx* c)
{
    cudaError_t e = cudaFuncSetAttribute(k_mlp_bf16, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(MlpSmem));
    if (e != cudaSuccess) return cuda_fail(c, e, "k_mlp_bf16 shared memory");
    e = cudaFuncSetAttribute(k_mlp_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM);
    if (e != cudaSuccess) return cuda_fail(c, e, "k_mlp_tc shared memory");
    e = cudaFuncSetAttribute(k_train_fb, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (ML_ND * ML_NH + ML_NH * ML_NH) * (int)sizeof(float));
    if (e != cudaSuccess) return cuda_fail(c, e, "k_train_fb shared memory");
    c->ml_attr = true;
    return NBG_OK;
}
