// Device-side building blocks of the Debye pair kernels, shared by the
// per-structure launches (debye_kernels.cu, adjoint_kernels.cu) and the
// persistent batch kernels (batch_kernels.cu).  Written from scratch for this
// project; see debye_kernels.cu for the overall scheme.
#pragma once
#include "rsx_internal.h"
#include "rsx_math.cuh"

namespace rsx {

// Reduce-scatter of QS per-lane values across the 32 lanes of a warp: on
// return v[0] of lane L holds the warp-wide sum of index (L & (QS-1)).
template <int QS>
__device__ __forceinline__ void warp_reduce_scatter(float (&v)[QS], int lane)
{
#pragma unroll
    for (int m = 16; m >= QS; m >>= 1) {
#pragma unroll
        for (int k = 0; k < QS; ++k)
            v[k] += __shfl_xor_sync(0xffffffffu, v[k], m);
    }
#pragma unroll
    for (int h = QS / 2; h >= 1; h >>= 1) {
        const bool up = (lane & h) != 0;
#pragma unroll
        for (int k = 0; k < h; ++k) {
            const float send = up ? v[k] : v[k + h];
            const float keep = up ? v[k + h] : v[k];
            v[k] = keep + __shfl_xor_sync(0xffffffffu, send, h);
        }
    }
}

// Warp-wide sums of 32 q values through shared memory: lane L stores its value
// of q index k at buf[k][L] (row stride kSumStride floats), then sums row L
// (the 32 lanes' values of q index L) with FP32x2 adds.  32 stores, 8 vector
// loads and 16 adds, against 31 shuffles, 31 adds and 62 selects for the
// shuffle reduce-scatter; both are bank-conflict free.  buf: 32 * kSumStride
// floats owned by the warp.
constexpr int kSumStride = 36;

template <typename F>
__device__ __forceinline__ float warp_sum_rows(F &&value_of, float *buf, int lane)
{
    __syncwarp();
#pragma unroll
    for (int k = 0; k < 32; ++k)
        buf[k * kSumStride + lane] = value_of(k);
    __syncwarp();
    const float4 *row = reinterpret_cast<const float4 *>(buf + lane * kSumStride);
    float4 v = row[0];
    float2 s0 = make_float2(v.x, v.y), s1 = make_float2(v.z, v.w);
#pragma unroll
    for (int j = 1; j < 8; ++j) {
        v = row[j];
        s0 = __fadd2_rn(s0, make_float2(v.x, v.y));
        s1 = __fadd2_rn(s1, make_float2(v.z, v.w));
    }
    s0 = __fadd2_rn(s0, s1);
    return s0.x + s0.y;
}

__device__ __forceinline__ void kahan_add(float &acc, float &comp, float x)
{
    const float y = x - comp;
    const float t = acc + y;
    comp = (t - acc) - y;
    acc = t;
}

// Distance terms of one pair: r and 1/r with r >= 1e-6 (coincident bodies
// then give sinc = 1, as the reference's device kernel does).  Both come from
// the hardware reciprocal square root y ~ 1/sqrt(r^2) (a few ulp), refined by
// one residual step each (Markstein's correction, with the residuals exact by
// FMA):  r = r0 + (r^2 - r0^2) y / 2 with r0 = r^2 y,  and  1/r = y + y (1 - r y).
// Each step squares the relative error, so the results are within about one
// ulp with no systematic offset.  The unrefined approximation does have one:
// over 1e10 pairs it shifts I(q) at high q by ~1e-4 relative (measured
// against the FP64 oracle at 50,000 and 200,000 bodies).  The refinement
// costs 5 FP32 operations, a third of the IEEE square root and reciprocal.
__device__ __forceinline__ void pair_r(const float4 &a, const float4 &b, float &r, float &rinv,
                                       float &dx, float &dy, float &dz)
{
    dx = b.x - a.x;
    dy = b.y - a.y;
    dz = b.z - a.z;
    float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
    r2 = fmaxf(r2, 1e-12f);
    const float y = rsqrtf(r2);
    const float r0 = r2 * y;
    r = fmaf(0.5f * y, fmaf(-r0, r0, r2), r0);
    rinv = fmaf(y, fmaf(-r, y, 1.0f), y);
}

// ----------------------------------------------------------------------------
// forward
// ----------------------------------------------------------------------------

// Seeds of the uniform-grid recurrence for one pair.  With x0 = q_0 r,
// theta = dq r and s_k = sin(x0 + k theta) / r (already scaled by `sc`):
//  * cos(theta) >= 0: Reinsch's modification of the second-order recurrence
//    (Reinsch; analysed by Gentleman, Comput. J. 12 (1969) 160-165):
//      d_{k+1} = d_k + lam s_k,  s_{k+1} = s_k + d_{k+1},
//      lam = -4 sin^2(theta/2),  d_0 = s_0 - s_{-1} = 2 sin(theta/2) cos(x0 - theta/2) / r
//    2 FP32 ops per step; it keeps relative accuracy for small theta where the
//    plain s_{k+1} = 2 cos(theta) s_k - s_{k-1} loses it (cos(theta) ~ 1).
//  * cos(theta) < 0 (coarse q grids): rotation of (s, c) by theta.
struct PairSeed {
    float s, d, lam; // Reinsch state (small) or s, c (rotation, in s, d)
    float sd, cd;    // rotation step (big only)
    bool big;
};

__device__ __forceinline__ PairSeed pair_seed(float q0, float dq, float r, float sc)
{
    PairSeed p;
    float s0, c0, sh, ch;
    sincos_prod(q0, r, s0, c0);                 // x0 = q0 r, exactly
    {
        const float th = dq * r;                // theta = dq r, exactly as th + th_lo
        const float th_lo = fmaf(dq, r, -th);
        sincos_rr2(0.5f * th, 0.5f * th_lo, sh, ch);
    }
    p.big = ch * ch < sh * sh;
    p.s = s0 * sc;
    if (!p.big) {
        p.lam = -4.0f * sh * sh;
        p.d = 2.0f * sh * fmaf(c0, ch, s0 * sh) * sc;
        p.sd = p.cd = 0.f;
    } else {
        p.d = c0 * sc;                    // cos(x0) / r
        p.sd = 2.0f * sh * ch;            // sin(theta)
        p.cd = fmaf(-2.0f * sh, sh, 1.0f); // cos(theta)
        p.lam = 0.f;
    }
    return p;
}

// One pair over the slab: S[k] += s_k (and SW[k] += w * s_k).
template <int QS, bool WATER>
__device__ __forceinline__ void pair_slab(PairSeed p, float wj, float (&S)[QS], float *SW)
{
    if (!p.big) {
        float s = p.s, d = p.d;
#pragma unroll
        for (int k = 0; k < QS; ++k) {
            S[k] += s;
            if (WATER)
                SW[k] = fmaf(wj, s, SW[k]);
            d = fmaf(p.lam, s, d);
            s += d;
        }
    } else {
        float s = p.s, c = p.d;
#pragma unroll
        for (int k = 0; k < QS; ++k) {
            S[k] += s;
            if (WATER)
                SW[k] = fmaf(wj, s, SW[k]);
            const float sn = fmaf(c, p.sd, s * p.cd);
            const float cn = fmaf(-s, p.sd, c * p.cd);
            s = sn;
            c = cn;
        }
    }
}

// Two pairs whose recurrences both use the Reinsch form, interleaved for ILP.
template <int QS>
__device__ __forceinline__ void pair2_slab(const PairSeed &a, const PairSeed &b, float (&S)[QS])
{
    float sa = a.s, da = a.d, sb = b.s, db = b.d;
#pragma unroll
    for (int k = 0; k < QS; ++k) {
        S[k] += sa + sb;
        da = fmaf(a.lam, sa, da);
        db = fmaf(b.lam, sb, db);
        sa += da;
        sb += db;
    }
}

template <int QS>
__device__ __forceinline__ void reduce_scatter_any(float (&v)[QS], int lane)
{
    if constexpr (QS <= 32) {
        warp_reduce_scatter<QS>(v, lane);
    } else {
        // QS = 64: two independent 32-wide scatters; lane L ends with index L
        // in v[0] and index 32 + L in v[32]
        float lo[32], hi[32];
#pragma unroll
        for (int k = 0; k < 32; ++k) {
            lo[k] = v[k];
            hi[k] = v[32 + k];
        }
        warp_reduce_scatter<32>(lo, lane);
        warp_reduce_scatter<32>(hi, lane);
        v[0] = lo[0];
        v[32] = hi[0];
    }
}

// ----------------------------------------------------------------------------
// forward, uniform q grid without water: wide slabs
// ----------------------------------------------------------------------------
//
// The per-pair seed (distance and 1/r, sin/cos(theta) and, past q = 0,
// sin/cos(q0 r)) costs as much as ~30 recurrence steps, so this form runs up
// to 192 q per seed.  Per J-block each thread sums its pairs in FP32 registers
// (S[m], q 2m and 2m + 1 in one float2);
// the warp then reduce-scatters S (lane L receives q index 32c + L of chunk c)
// and adds it to FP64 lane accumulators, so no per-thread compensated
// accumulators have to be kept for QS q values.  (Summing through shared
// memory instead, as the delta kernel does for its small tiles, took 0.7 %
// fewer instructions here but ran 3 % slower at 2 CTAs per SM.)

template <int QS>
struct WideSlab {
    static constexpr int QP = (QS + 31) / 32 * 32; // padded to whole warps
    static constexpr int NR = QP / 32;             // q values per lane after the scatter
};

// Seed of the wide path: Reinsch's recurrence in paired steps.  The q values
// of a slab are taken two at a time: the even ones (k = 2m) and the odd ones
// (k = 2m + 1) form two sequences with the step 2 theta (theta = dq r), packed
// in one float2 so that every FP32x2 instruction (__ffma2_rn, __fadd2_rn)
// advances both.  The FP32 lane work stays at 3 operations per pair*q, but
// the issue slots are halved: the scalar loop is issue-bound (a measured 77 %
// of the FMA rate in a register-resident test), the paired one runs at the
// FMA rate.  Reinsch's form, with lam = -4 sin^2(theta) (the half angle of
// the step 2 theta):
//     d_{m+1} = d_m + lam s_m,   s_{m+1} = s_m + d_{m+1},
// seeded with d_0 = s_0 - s_{-1}, the previous element of the same sequence:
//     even: sin(x0) - sin(x0 - 2 theta)     = 2 sin(theta) cos(x0 - theta)
//     odd:  sin(x0 + theta) - sin(x0 - theta) = 2 sin(theta) cos(x0).
// The form is accurate while cos^2(theta) >= sin^2(theta).  Elsewhere (theta
// mod pi in (pi/4, 3 pi/4): far-apart bodies on coarse grids) both sequences
// run instead on t_m = (-1)^m s_m, whose step 2 theta - pi is back in range:
//     lam = -4 cos^2(theta),
//     d_0 = 2 cos(theta) sin(x0 - theta) (even),  2 cos(theta) sin(x0) (odd),
// and odd m are accumulated with the sign sg = -1.  So every pair steps an
// angle of magnitude <= pi/2 with the same operations, and no warp diverges
// on far pairs.
struct WideSeed {
    float2 s, d; // (even, odd) t_0 / r and d_0 / r
    float l, sg; // lam, sign of the odd steps (+1 or -1)
};

// `small_theta` (uniform over the launch) promises |theta| < pi/4 for every
// pair, where the reduction is the identity (sincos_small2 gives sincos_rr2's
// results bit for bit) and every sign is +1.
__device__ __forceinline__ WideSeed wide_seed(float q0, float dq, float r, float sc,
                                              bool small_theta = false)
{
    float s0, c0, st, ct;
    const float th = dq * r;
    const float th_lo = fmaf(dq, r, -th);
    if (small_theta)
        sincos_small2(th, th_lo, st, ct);
    else
        sincos_rr2(th, th_lo, st, ct);
    // x0 = q0 r: 0 at q0 = 0; at q0 = dq (the first q of a past_q0 view) the
    // step's own sin/cos, sincos_prod(dq, r) bit for bit.  (This form, one
    // branch with selects, measured fastest of three on the two-slab chains
    // and the batched chains; see wide_seed_x0_first.)
    if (q0 != 0.f && q0 != dq) {
        sincos_prod(q0, r, s0, c0);
    } else {
        const bool zero = q0 == 0.f;
        s0 = zero ? 0.f : st;
        c0 = zero ? 1.f : ct;
    }
    WideSeed p;
    p.s = make_float2(s0 * sc, fmaf(s0, ct, c0 * st) * sc); // sin(x0), sin(x0 + theta)
    if (small_theta || ct * ct >= st * st) { // |theta| < pi/4: never folded
        p.l = -4.0f * st * st;
        const float g = 2.0f * st * sc;
        p.d = make_float2(g * fmaf(c0, ct, s0 * st), g * c0);
        p.sg = 1.0f;
    } else {
        p.l = -4.0f * ct * ct;
        const float g = 2.0f * ct * sc;
        p.d = make_float2(g * fmaf(s0, ct, -c0 * st), g * s0);
        p.sg = -1.0f;
    }
    return p;
}

// The same seed with sin/cos(x0) evaluated before sin/cos(theta), bit for bit
// the same values.  Which order the compiler schedules better depends on the
// kernel around it: measured on the single-structure chains with a tail slab
// (forward_chain_kernel, QT > 0) at 201 q, this one took 4.19 against 4.42 ms,
// while the two-slab chains and the batched chains ran 0.2-0.9 % faster with
// wide_seed.
__device__ __forceinline__ WideSeed wide_seed_x0_first(float q0, float dq, float r, float sc,
                                                       bool small_theta = false)
{
    float s0 = 0.f, c0 = 1.f, st, ct;
    if (q0 != 0.f && q0 != dq)
        sincos_prod(q0, r, s0, c0);
    const float th = dq * r;
    const float th_lo = fmaf(dq, r, -th);
    if (small_theta)
        sincos_small2(th, th_lo, st, ct);
    else
        sincos_rr2(th, th_lo, st, ct);
    if (q0 == dq && q0 != 0.f) {
        s0 = st;
        c0 = ct;
    }
    WideSeed p;
    p.s = make_float2(s0 * sc, fmaf(s0, ct, c0 * st) * sc);
    if (small_theta || ct * ct >= st * st) {
        p.l = -4.0f * st * st;
        const float g = 2.0f * st * sc;
        p.d = make_float2(g * fmaf(c0, ct, s0 * st), g * c0);
        p.sg = 1.0f;
    } else {
        p.l = -4.0f * ct * ct;
        const float g = 2.0f * ct * sc;
        p.d = make_float2(g * fmaf(s0, ct, -c0 * st), g * s0);
        p.sg = -1.0f;
    }
    return p;
}

__device__ __forceinline__ float2 splat2(float x) { return make_float2(x, x); }

// A chain's state between two slabs keeps the sign of its odd steps (sg, +1
// or -1) in the sign bit of lam, which is -4 x^2 (sign bit set, -0.0
// included): a clear sign bit stands for sg = -1.
__device__ __forceinline__ float pack_lam_sign(float l, float sg) { return sg > 0.f ? l : -l; }
__device__ __forceinline__ void unpack_lam_sign(float x, float &l, float &sg)
{
    sg = signbit(x) ? 1.f : -1.f;
    l = -fabsf(x);
}

// Two pairs, interleaved for ILP (the hot loop: per paired step of both
// pairs 6 FP32x2 instructions = 12 lane-ops for 4 pair*q).  S[m] holds
// (q_{2m}, q_{2m+1}).  SIGNED adds the odd steps with the pairs' signs;
// warps whose pairs all have sign +1 (compact structures: all of them) take
// the plain adds.
// The chains' states after the QS q are left in a.s, a.d and b.s, b.d, so a
// following slab can continue them without a new seed (QS / 2 must then be
// even for the signs of the odd steps to line up).
template <int QS, int QH, bool SIGNED>
__device__ __forceinline__ void wide_pair2_carry(WideSeed &a, WideSeed &b, float2 (&S)[QH])
{
    float2 sa = a.s, da = a.d, sb = b.s, db = b.d;
    const float2 la = splat2(a.l), lb = splat2(b.l);
#pragma unroll
    for (int m = 0; m < QS / 2; ++m) {
        if (SIGNED && (m & 1))
            S[m] = __ffma2_rn(splat2(a.sg), sa, __ffma2_rn(splat2(b.sg), sb, S[m]));
        else
            S[m] = __fadd2_rn(S[m], __fadd2_rn(sa, sb));
        da = __ffma2_rn(la, sa, da);
        db = __ffma2_rn(lb, sb, db);
        sa = __fadd2_rn(sa, da);
        sb = __fadd2_rn(sb, db);
    }
    a.s = sa;
    a.d = da;
    b.s = sb;
    b.d = db;
}

template <int QS, int QH, bool SIGNED>
__device__ __forceinline__ void wide_pair2_body(const WideSeed &a, const WideSeed &b,
                                                float2 (&S)[QH])
{
    WideSeed x = a, y = b;
    wide_pair2_carry<QS, QH, SIGNED>(x, y, S);
}

template <int QS, int QH>
__device__ __forceinline__ void wide_pair2(const WideSeed &a, const WideSeed &b, float2 (&S)[QH])
{
    if (__any_sync(0xffffffffu, a.sg < 0.f || b.sg < 0.f))
        wide_pair2_body<QS, QH, true>(a, b, S);
    else
        wide_pair2_body<QS, QH, false>(a, b, S);
}

// Four pairs: more independent chains per warp for when few warps fit on an SM.
template <int QS, int QH, bool SIGNED>
__device__ __forceinline__ void wide_pair4_body(const WideSeed &a, const WideSeed &b,
                                                const WideSeed &c, const WideSeed &e,
                                                float2 (&S)[QH])
{
    float2 sa = a.s, da = a.d, sb = b.s, db = b.d, sc = c.s, dc = c.d, se = e.s, de = e.d;
    const float2 la = splat2(a.l), lb = splat2(b.l), lc = splat2(c.l), le = splat2(e.l);
#pragma unroll
    for (int m = 0; m < QS / 2; ++m) {
        if (SIGNED && (m & 1))
            S[m] = __ffma2_rn(splat2(a.sg), sa,
                              __ffma2_rn(splat2(b.sg), sb,
                                         __ffma2_rn(splat2(c.sg), sc,
                                                    __ffma2_rn(splat2(e.sg), se, S[m]))));
        else
            S[m] = __fadd2_rn(S[m], __fadd2_rn(__fadd2_rn(sa, sb), __fadd2_rn(sc, se)));
        da = __ffma2_rn(la, sa, da);
        db = __ffma2_rn(lb, sb, db);
        dc = __ffma2_rn(lc, sc, dc);
        de = __ffma2_rn(le, se, de);
        sa = __fadd2_rn(sa, da);
        sb = __fadd2_rn(sb, db);
        sc = __fadd2_rn(sc, dc);
        se = __fadd2_rn(se, de);
    }
}

template <int QS, int QH>
__device__ __forceinline__ void wide_pair4(const WideSeed &a, const WideSeed &b, const WideSeed &c,
                                           const WideSeed &e, float2 (&S)[QH])
{
    if (__any_sync(0xffffffffu, a.sg < 0.f || b.sg < 0.f || c.sg < 0.f || e.sg < 0.f))
        wide_pair4_body<QS, QH, true>(a, b, c, e, S);
    else
        wide_pair4_body<QS, QH, false>(a, b, c, e, S);
}

template <int QS, int QH>
__device__ __forceinline__ void wide_pair1(const WideSeed &p, float2 (&S)[QH])
{
    float2 s = p.s, d = p.d;
    const float2 l = splat2(p.l), g = splat2(p.sg);
#pragma unroll
    for (int m = 0; m < QS / 2; ++m) {
        S[m] = (m & 1) ? __ffma2_rn(g, s, S[m]) : __fadd2_rn(S[m], s);
        d = __ffma2_rn(l, s, d);
        s = __fadd2_rn(s, d);
    }
}

// Value of q index k of a paired accumulator array.
template <int QH>
__device__ __forceinline__ float pair_at(const float2 (&S)[QH], int k)
{
    return (k & 1) ? S[k >> 1].y : S[k >> 1].x;
}

// Forward pair sums of one work item for q values [k0, k0 + QS) on a uniform
// grid without water; writes partial[k][item_idx] as forward_item does.
// SIGNED = false: the launch promises small theta (small_theta level 2: every
// pair has |theta| < pi/4, so every sign is +1), and the pair loop keeps only
// the plain adds.
template <int QS, int IL, bool SIGNED = true>
__device__ __forceinline__ void forward_wide_item(const DebyeArgs &a, int item_idx, int k0)
{
    constexpr int QP = WideSlab<QS>::QP, NR = WideSlab<QS>::NR;
    __shared__ float4 s_pos[kBlockAtoms];
    __shared__ double s_red[kBlockAtoms / 32][QP];

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    __syncthreads(); // a previous item of this CTA may still read shared memory
    const PairItem it = a.items[item_idx];
    const BlockDesc bi = a.blocks[it.bi];
    const int tj = a.blocks[it.bj_begin].type;
    const int i = bi.start + tid;
    const bool valid_i = tid < bi.len;
    const float4 pi = valid_i ? a.pos[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float q0 = a.q[k0];
    const float dq = a.dq;
    const bool small_th = !SIGNED || a.small_theta >= 2;

    double acc[NR];
#pragma unroll
    for (int c = 0; c < NR; ++c)
        acc[c] = 0.0;

    for (int b = it.bj_begin; b < it.bj_end; ++b) {
        const BlockDesc bj = a.blocks[b];
        __syncthreads();
        if (tid < bj.len)
            s_pos[tid] = a.pos[bj.start + tid];
        __syncthreads();
        const bool diag = (b == it.bi);
        float2 S[QP / 2];
#pragma unroll
        for (int m = 0; m < QP / 2; ++m)
            S[m] = make_float2(0.f, 0.f);
        int jj = 0;
        if (IL == 4) {
            for (; jj + 3 < bj.len; jj += 4) {
                WideSeed p[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    float r, ri, dx, dy, dz;
                    pair_r(pi, s_pos[jj + u], r, ri, dx, dy, dz);
                    const bool use = valid_i && (!diag || jj + u > tid);
                    p[u] = wide_seed(q0, dq, r, use ? ri : 0.f, small_th);
                }
                if constexpr (SIGNED)
                    wide_pair4<QS, QP / 2>(p[0], p[1], p[2], p[3], S);
                else
                    wide_pair4_body<QS, QP / 2, false>(p[0], p[1], p[2], p[3], S);
            }
        }
        for (; jj + 1 < bj.len; jj += 2) {
            float r1, ri1, r2, ri2, dx, dy, dz;
            pair_r(pi, s_pos[jj], r1, ri1, dx, dy, dz);
            pair_r(pi, s_pos[jj + 1], r2, ri2, dx, dy, dz);
            const bool u1 = valid_i && (!diag || jj > tid);
            const bool u2 = valid_i && (!diag || jj + 1 > tid);
            const WideSeed p1 = wide_seed(q0, dq, r1, u1 ? ri1 : 0.f, small_th);
            const WideSeed p2 = wide_seed(q0, dq, r2, u2 ? ri2 : 0.f, small_th);
            if constexpr (SIGNED)
                wide_pair2<QS, QP / 2>(p1, p2, S);
            else
                wide_pair2_body<QS, QP / 2, false>(p1, p2, S);
        }
        if (jj < bj.len) {
            float r, rinv, dx, dy, dz;
            pair_r(pi, s_pos[jj], r, rinv, dx, dy, dz);
            const bool use = valid_i && (!diag || jj > tid);
            wide_pair1<QS, QP / 2>(wide_seed(q0, dq, r, use ? rinv : 0.f, small_th), S);
        }
#pragma unroll
        for (int c = 0; c < NR; ++c) {
            float v[32];
#pragma unroll
            for (int k = 0; k < 32; ++k)
                v[k] = pair_at(S, 32 * c + k);
            warp_reduce_scatter<32>(v, lane);
            acc[c] += (double)v[0];
        }
    }

#pragma unroll
    for (int c = 0; c < NR; ++c)
        s_red[warp][32 * c + lane] = acc[c];
    __syncthreads();
    for (int k = tid; k < QS; k += kBlockAtoms) {
        const int kk = k0 + k;
        if (kk >= a.n_q)
            continue;
        double s = 0.0;
#pragma unroll
        for (int w = 0; w < kBlockAtoms / 32; ++w)
            s += s_red[w][k];
        const double fi = a.ff[(size_t)kk * a.n_types + bi.type];
        const double fj = a.ff[(size_t)kk * a.n_types + tj];
        a.partial[(size_t)kk * a.n_items + item_idx] = s * fi * fj;
    }
}

// ----------------------------------------------------------------------------
// forward, uniform q grid with the implicit water term: wide slabs
// ----------------------------------------------------------------------------
//
// With water every body's factor is f~_b(q) = f_t(q) + w rsasa_b f_w(q), so a
// pair term is f~_i f~_j sin(q r)/r.  Per J-block a thread accumulates
// U(q) = sum_j f~_j(q) sin(q r_ij)/r_ij: the coefficient of pair j at q 2m and
// 2m + 1 is one FP32x2 FMA from a per-item table row (f_tj and w f_w at both
// q) and the pair's rsasa, and the sum one more, so a pair*q costs 4 FP32
// lane-ops with the recurrence.  f~_i(q) multiplies U once per J-block,
// before the warp reduce-scatter (it differs from lane to lane).

// Two pairs with their rsasa values ra, rb; fq[m] = (f_tj(q_2m), f_tj(q_2m+1),
// w f_w(q_2m), w f_w(q_2m+1)).  SIGNED multiplies the odd steps' coefficients
// by the pairs' signs.
template <int QS, int QH, bool SIGNED>
__device__ __forceinline__ void wide_water_pair2_body(const WideSeed &a, const WideSeed &b,
                                                      float ra, float rb, const float4 *fq,
                                                      float2 (&S)[QH])
{
    float2 sa = a.s, da = a.d, sb = b.s, db = b.d;
    const float2 la = splat2(a.l), lb = splat2(b.l), rsa = splat2(ra), rsb = splat2(rb);
#pragma unroll
    for (int m = 0; m < QS / 2; ++m) {
        const float4 f = fq[m];
        const float2 fj = make_float2(f.x, f.y), fw = make_float2(f.z, f.w);
        float2 ca = __ffma2_rn(fw, rsa, fj), cb = __ffma2_rn(fw, rsb, fj);
        if (SIGNED && (m & 1)) {
            ca = __fmul2_rn(splat2(a.sg), ca);
            cb = __fmul2_rn(splat2(b.sg), cb);
        }
        S[m] = __ffma2_rn(ca, sa, __ffma2_rn(cb, sb, S[m]));
        da = __ffma2_rn(la, sa, da);
        db = __ffma2_rn(lb, sb, db);
        sa = __fadd2_rn(sa, da);
        sb = __fadd2_rn(sb, db);
    }
}

template <int QS, int QH>
__device__ __forceinline__ void wide_water_pair2(const WideSeed &a, const WideSeed &b, float ra,
                                                 float rb, const float4 *fq, float2 (&S)[QH])
{
    if (__any_sync(0xffffffffu, a.sg < 0.f || b.sg < 0.f))
        wide_water_pair2_body<QS, QH, true>(a, b, ra, rb, fq, S);
    else
        wide_water_pair2_body<QS, QH, false>(a, b, ra, rb, fq, S);
}

template <int QS, int QH>
__device__ __forceinline__ void wide_water_pair1(const WideSeed &p, float rp, const float4 *fq,
                                                 float2 (&S)[QH])
{
    float2 s = p.s, d = p.d;
    const float2 l = splat2(p.l), rs = splat2(rp);
#pragma unroll
    for (int m = 0; m < QS / 2; ++m) {
        const float4 f = fq[m];
        float2 c = __ffma2_rn(make_float2(f.z, f.w), rs, make_float2(f.x, f.y));
        if (m & 1)
            c = __fmul2_rn(splat2(p.sg), c);
        S[m] = __ffma2_rn(c, s, S[m]);
        d = __ffma2_rn(l, s, d);
        s = __fadd2_rn(s, d);
    }
}

// Forward pair sums with water of one work item for q values [k0, k0 + QS) on
// a uniform grid; writes partial[k][item_idx] = sum over the item's pairs of
// f~_i f~_j sin(q_k r)/r (the factors included, as forward_item<QS, U, true>
// does).  SIGNED as in forward_wide_item.
template <int QS, bool SIGNED = true>
__device__ __forceinline__ void forward_wide_water_item(const DebyeArgs &a, int item_idx, int k0)
{
    constexpr int QP = WideSlab<QS>::QP, NR = WideSlab<QS>::NR;
    __shared__ float4 s_pos[kBlockAtoms];
    __shared__ float s_rs[kBlockAtoms];
    __shared__ float4 s_fq[QP / 2];
    __shared__ float s_fi[QP], s_fw[QP];
    __shared__ double s_red[kBlockAtoms / 32][QP];

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    __syncthreads(); // a previous item of this CTA may still read shared memory
    const PairItem it = a.items[item_idx];
    const BlockDesc bi = a.blocks[it.bi];
    const int tj = a.blocks[it.bj_begin].type;
    for (int k = tid; k < QP; k += kBlockAtoms) {
        const int kk = k0 + k;
        const bool in = k < QS && kk < a.n_q;
        const float *row = a.ff + (size_t)(in ? kk : 0) * a.n_types;
        s_fi[k] = in ? row[bi.type] : 0.f;
        s_fw[k] = in ? a.water_weight * row[a.water_index] : 0.f;
        const float fj = in ? row[tj] : 0.f;
        // the table row of step m = k / 2 holds both q of the step
        float *fq = reinterpret_cast<float *>(&s_fq[k >> 1]);
        fq[k & 1] = fj;
        fq[2 + (k & 1)] = s_fw[k];
    }
    const int i = bi.start + tid;
    const bool valid_i = tid < bi.len;
    const float4 pi = valid_i ? a.pos[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float rs_i = valid_i ? a.rsasa[i] : 0.f;
    const float q0 = a.q[k0];
    const float dq = a.dq;
    const bool small_th = !SIGNED || a.small_theta >= 2;

    double acc[NR];
#pragma unroll
    for (int c = 0; c < NR; ++c)
        acc[c] = 0.0;

    for (int b = it.bj_begin; b < it.bj_end; ++b) {
        const BlockDesc bj = a.blocks[b];
        __syncthreads();
        if (tid < bj.len) {
            s_pos[tid] = a.pos[bj.start + tid];
            s_rs[tid] = a.rsasa[bj.start + tid];
        }
        __syncthreads();
        const bool diag = (b == it.bi);
        float2 S[QP / 2];
#pragma unroll
        for (int m = 0; m < QP / 2; ++m)
            S[m] = make_float2(0.f, 0.f);
        int jj = 0;
        for (; jj + 1 < bj.len; jj += 2) {
            // the table rows are the same for every pair: an offset the
            // compiler cannot see through keeps it from hoisting all of them
            // into registers (one shared load per step is the intent)
            int fo = 0;
            asm volatile("" : "+r"(fo));
            float r1, ri1, r2, ri2, dx, dy, dz;
            pair_r(pi, s_pos[jj], r1, ri1, dx, dy, dz);
            pair_r(pi, s_pos[jj + 1], r2, ri2, dx, dy, dz);
            const bool u1 = valid_i && (!diag || jj > tid);
            const bool u2 = valid_i && (!diag || jj + 1 > tid);
            const WideSeed p1 = wide_seed(q0, dq, r1, u1 ? ri1 : 0.f, small_th);
            const WideSeed p2 = wide_seed(q0, dq, r2, u2 ? ri2 : 0.f, small_th);
            if constexpr (SIGNED)
                wide_water_pair2<QS, QP / 2>(p1, p2, s_rs[jj], s_rs[jj + 1], s_fq + fo, S);
            else
                wide_water_pair2_body<QS, QP / 2, false>(p1, p2, s_rs[jj], s_rs[jj + 1],
                                                         s_fq + fo, S);
        }
        if (jj < bj.len) {
            int fo = 0;
            asm volatile("" : "+r"(fo));
            float r, rinv, dx, dy, dz;
            pair_r(pi, s_pos[jj], r, rinv, dx, dy, dz);
            const bool use = valid_i && (!diag || jj > tid);
            wide_water_pair1<QS, QP / 2>(wide_seed(q0, dq, r, use ? rinv : 0.f, small_th),
                                         s_rs[jj], s_fq + fo, S);
        }
#pragma unroll
        for (int c = 0; c < NR; ++c) {
            float v[32];
#pragma unroll
            for (int k = 0; k < 32; ++k) {
                const int kq = 32 * c + k;
                v[k] = fmaf(rs_i, s_fw[kq], s_fi[kq]) * pair_at(S, kq);
            }
            warp_reduce_scatter<32>(v, lane);
            acc[c] += (double)v[0];
        }
    }

#pragma unroll
    for (int c = 0; c < NR; ++c)
        s_red[warp][32 * c + lane] = acc[c];
    __syncthreads();
    for (int k = tid; k < QS; k += kBlockAtoms) {
        const int kk = k0 + k;
        if (kk >= a.n_q)
            continue;
        double s = 0.0;
#pragma unroll
        for (int w = 0; w < kBlockAtoms / 32; ++w)
            s += s_red[w][k];
        a.partial[(size_t)kk * a.n_items + item_idx] = s;
    }
}

// Forward pair sums of one work item for q values [k0, k0 + QS): writes
// partial[k][item_idx] = sum over the item's pairs of f_i f_j sin(q_k r)/r.
// Called once per CTA by the grid kernel and repeatedly by the persistent
// batch kernel (hence the leading barrier).
template <int QS, bool UNIFORM, bool WATER>
__device__ __forceinline__ void forward_item(const DebyeArgs &a, int item_idx, int k0)
{
    __shared__ float4 s_pos[kBlockAtoms];
    __shared__ float s_rs[WATER ? kBlockAtoms : 1];
    __shared__ float s_q[QS], s_fi[QS], s_fj[QS], s_fw[QS];
    __shared__ float s_comp[QS][kBlockAtoms];                 // Kahan terms, per thread
    __shared__ float s_compw[WATER ? QS : 1][kBlockAtoms];
    __shared__ double s_red[kBlockAtoms / 32][QS];

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    __syncthreads(); // a previous item of this CTA may still read shared memory
    const PairItem it = a.items[item_idx];
    const BlockDesc bi = a.blocks[it.bi];
    const int tj = a.blocks[it.bj_begin].type;
    for (int k = tid; k < QS; k += kBlockAtoms) {
        const int kk = k0 + k;
        const bool in = kk < a.n_q;
        s_q[k] = in ? a.q[kk] : 0.f;
        s_fi[k] = in ? a.ff[(size_t)kk * a.n_types + bi.type] : 0.f;
        s_fj[k] = in ? a.ff[(size_t)kk * a.n_types + tj] : 0.f;
        s_fw[k] = (WATER && in) ? a.water_weight * a.ff[(size_t)kk * a.n_types + a.water_index]
                                : 0.f;
    }
    const int i = bi.start + tid;
    const bool valid_i = tid < bi.len;
    const float4 pi = valid_i ? a.pos[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float rs_i = (WATER && valid_i) ? a.rsasa[i] : 0.f;

    float acc[QS], accw[WATER ? QS : 1];
#pragma unroll
    for (int k = 0; k < QS; ++k) {
        acc[k] = 0.f;
        s_comp[k][tid] = 0.f;
        if (WATER) {
            accw[k] = 0.f;
            s_compw[k][tid] = 0.f;
        }
    }
    __syncthreads();
    const float q0 = s_q[0];
    const float dq = a.dq;

    for (int b = it.bj_begin; b < it.bj_end; ++b) {
        const BlockDesc bj = a.blocks[b];
        __syncthreads();
        if (tid < bj.len) {
            s_pos[tid] = a.pos[bj.start + tid];
            if (WATER)
                s_rs[tid] = a.rsasa[bj.start + tid];
        }
        __syncthreads();
        const bool diag = (b == it.bi);
        float S[QS], SW[WATER ? QS : 1];
#pragma unroll
        for (int k = 0; k < QS; ++k) {
            S[k] = 0.f;
            if (WATER)
                SW[k] = 0.f;
        }
        int jj = 0;
        if (UNIFORM && !WATER) {
            for (; jj + 1 < bj.len; jj += 2) {
                float r1, ri1, r2, ri2, dx, dy, dz;
                pair_r(pi, s_pos[jj], r1, ri1, dx, dy, dz);
                pair_r(pi, s_pos[jj + 1], r2, ri2, dx, dy, dz);
                const bool u1 = valid_i && (!diag || jj > tid);
                const bool u2 = valid_i && (!diag || jj + 1 > tid);
                const PairSeed p1 = pair_seed(q0, dq, r1, u1 ? ri1 : 0.f);
                const PairSeed p2 = pair_seed(q0, dq, r2, u2 ? ri2 : 0.f);
                if (!p1.big && !p2.big) {
                    pair2_slab<QS>(p1, p2, S);
                } else {
                    pair_slab<QS, false>(p1, 0.f, S, SW);
                    pair_slab<QS, false>(p2, 0.f, S, SW);
                }
            }
        }
        for (; jj < bj.len; ++jj) {
            float r, rinv, dx, dy, dz;
            pair_r(pi, s_pos[jj], r, rinv, dx, dy, dz);
            const bool use = valid_i && (!diag || jj > tid);
            const float sc = use ? rinv : 0.f;
            const float rs_j = WATER ? s_rs[jj] : 0.f;
            if (UNIFORM) {
                const PairSeed p = pair_seed(q0, dq, r, sc);
                pair_slab<QS, WATER>(p, rs_j, S, SW);
            } else {
#pragma unroll
                for (int k = 0; k < QS; ++k) {
                    float sk, ck;
                    sincos_prod(s_q[k], r, sk, ck);
                    const float v = sk * sc;
                    S[k] += v;
                    if (WATER)
                        SW[k] = fmaf(rs_j, v, SW[k]);
                }
            }
        }
#pragma unroll
        for (int k = 0; k < QS; ++k) {
            float c = s_comp[k][tid];
            kahan_add(acc[k], c, S[k]);
            s_comp[k][tid] = c;
            if (WATER) {
                float cw = s_compw[k][tid];
                kahan_add(accw[k], cw, SW[k]);
                s_compw[k][tid] = cw;
            }
        }
    }

    float v[QS];
#pragma unroll
    for (int k = 0; k < QS; ++k) {
        const float tot = acc[k] - s_comp[k][tid];
        if (WATER) {
            const float fi = fmaf(rs_i, s_fw[k], s_fi[k]);
            const float totw = accw[k] - s_compw[k][tid];
            v[k] = valid_i ? fi * fmaf(s_fj[k], tot, s_fw[k] * totw) : 0.f;
        } else {
            v[k] = valid_i ? tot : 0.f;
        }
    }
    reduce_scatter_any<QS>(v, lane);
    if (QS <= 32) {
        if (lane < QS)
            s_red[warp][lane] = (double)v[0];
    } else {
        s_red[warp][lane] = (double)v[0];
        s_red[warp][32 + lane] = (double)v[QS > 32 ? 32 : 0];
    }
    __syncthreads();
    for (int k = tid; k < QS; k += kBlockAtoms) {
        if (k0 + k >= a.n_q)
            continue;
        double s = 0.0;
#pragma unroll
        for (int w = 0; w < kBlockAtoms / 32; ++w)
            s += s_red[w][k];
        if (!WATER)
            s *= (double)s_fi[k] * (double)s_fj[k];
        a.partial[(size_t)(k0 + k) * a.n_items + item_idx] = s;
    }
}

// ----------------------------------------------------------------------------
// adjoint, uniform q grid without water
// ----------------------------------------------------------------------------
//
// Per pair the gradient needs A = sum_k alpha_k cos(x_k) and
// B = sum_k beta_k sin(x_k), x_k = q_k r, alpha_k = lambda_k f_i f_j,
// beta_k = alpha_k / q_k.  Both come from one two-term recurrence, the
// "magic circle" form of the sine/cosine oscillator:
//     e_{k+1} = e_k - a s_k,   s_{k+1} = s_k + a e_{k+1},   a = 2 sin(theta/2)
// with s_k = sin(x_k) and e_k = cos(x_k - theta/2) (exact in real arithmetic:
// cos(x + h) - cos(x - h) = -2 sin(x) sin(h), sin(x + 2h) - sin(x) =
// 2 cos(x + h) sin(h)).  Its errors stay at the rounding level for small theta,
// where the plain rotation's cos(theta) ~ 1 loses them.  Since
// cos(x_k) = (e_k + e_{k+1}) / (2 cos(theta/2)), summation by parts gives
//     A = sum_{m=0..L} delta_m e_m / (2 cos(theta/2)),
//     delta_m = alpha_m + alpha_{m-1}   (alpha outside the slab = 0),
// so a pair costs four FMAs per q: two for the recurrence and one for each
// sum.  Pairs step two at a time, packed in float2 lanes, so each FP32x2
// instruction (__ffma2_rn) advances both: the same lane work in half the
// issue slots.  The recurrence is reseeded from sin/cos(q_0 r) every kAdjSlab
// q.  Pairs with theta > pi/2 (cos(theta/2)^2 < 1/2, far-apart bodies on
// coarse grids) take the rotation form with alpha directly.

constexpr int kAdjSlab = 256;   // q values between reseeds
constexpr int kAdjStride = 257; // table entries per slab (delta has L + 1)

// Table entry m of slab sl: tab = (delta_m, delta_m, beta_m, beta_m) (each
// coefficient twice, the operand of a paired instruction) and tab_a = alpha_m
// (the rotation form's cosine coefficient).
__device__ __forceinline__ void adjoint_uniform_table(const DebyeArgs &a, float4 *tab,
                                                      float *tab_a, int n_slabs,
                                                      const float *lambda, int ti, int tj)
{
    const int n = n_slabs * kAdjStride;
    for (int idx = threadIdx.x; idx < n; idx += blockDim.x) {
        const int sl = idx / kAdjStride, m = idx - sl * kAdjStride;
        const int kb = sl * kAdjSlab;
        const int len = min(kAdjSlab, a.n_q - kb);
        auto alpha = [&](int k, float *beta) {
            // alpha_k, and beta_k = alpha_k / q_k (0 at q = 0, where d sinc/dr = 0)
            if (k < 0 || k >= len) {
                *beta = 0.f;
                return 0.f;
            }
            const int kk = kb + k;
            const float qk = a.q[kk];
            if (qk == 0.f) {
                *beta = 0.f;
                return 0.f;
            }
            const float al =
                lambda[kk] * a.ff[(size_t)kk * a.n_types + ti] * a.ff[(size_t)kk * a.n_types + tj];
            *beta = al / qk;
            return al;
        };
        float b0, bm1;
        const float a0 = alpha(m, &b0);
        const float am1 = alpha(m - 1, &bm1);
        tab[idx] = make_float4(a0 + am1, a0 + am1, b0, b0);
        tab_a[idx] = a0;
    }
}

// One pair over one slab of L q values (L a multiple of 8): P += sum delta e,
// Q += sum beta s.
__device__ __forceinline__ void adj_circle_slab(const float4 *t, int L, float s, float e, float ac,
                                                float &P, float &Q)
{
    for (int c = 0; c < L; c += 8) {
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const float4 cf = t[c + u];
            P = fmaf(cf.x, e, P);
            Q = fmaf(cf.z, s, Q);
            e = fmaf(-ac, s, e);
            s = fmaf(ac, e, s);
        }
    }
    P = fmaf(t[L].x, e, P);
}

// NP float2 lanes of two pairs each (all on the magic-circle form): one table
// load feeds all of them.  The recurrence steps in FP32x2 instructions; the
// two sums stay scalar FMAs (measured 3 % faster at 8 pairs per step than
// paired sums, whose three fresh 64-bit operands per instruction slow issue).
template <int NP>
__device__ __forceinline__ void adj_circle_slab_paired(const float4 *t, int L, float2 (&s)[NP],
                                                       float2 (&e)[NP], const float2 (&ac)[NP],
                                                       float2 (&P)[NP], float2 (&Q)[NP])
{
    float2 nac[NP];
#pragma unroll
    for (int v = 0; v < NP; ++v)
        nac[v] = make_float2(-ac[v].x, -ac[v].y);
    for (int c = 0; c < L; c += 8) {
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const float4 cf = t[c + u];
            const float2 dd = make_float2(cf.x, cf.y), bb = make_float2(cf.z, cf.w);
#pragma unroll
            for (int v = 0; v < NP; ++v) {
                P[v].x = fmaf(dd.x, e[v].x, P[v].x);
                P[v].y = fmaf(dd.x, e[v].y, P[v].y);
                Q[v].x = fmaf(bb.x, s[v].x, Q[v].x);
                Q[v].y = fmaf(bb.x, s[v].y, Q[v].y);
            }
#pragma unroll
            for (int v = 0; v < NP; ++v)
                e[v] = __ffma2_rn(nac[v], s[v], e[v]);
#pragma unroll
            for (int v = 0; v < NP; ++v)
                s[v] = __ffma2_rn(ac[v], e[v], s[v]);
        }
    }
    const float4 cf = t[L];
    const float2 dd = make_float2(cf.x, cf.y);
#pragma unroll
    for (int v = 0; v < NP; ++v)
        P[v] = __ffma2_rn(dd, e[v], P[v]);
}

// Rotation form for one pair over one slab: A += sum alpha cos, B += sum beta sin.
__device__ __forceinline__ void adj_rotate_slab(const float4 *t, const float *ta, int L, float s,
                                                float c, float sd, float cd, float &A, float &B)
{
    for (int k = 0; k < L; ++k) {
        A = fmaf(ta[k], c, A);
        B = fmaf(t[k].z, s, B);
        const float sn = fmaf(c, sd, s * cd);
        const float cn = fmaf(-s, sd, c * cd);
        s = sn;
        c = cn;
    }
}

// Per-pair constants of the uniform adjoint.
struct AdjPair {
    float r, rinv, dx, dy, dz;
    float sh, ch; // sin, cos of theta / 2
    bool circle;  // magic-circle form (theta <= pi/2)
};

// SMALL: the launch promises |theta/2| < pi/4 for every pair, so the
// reduction-free sincos applies (a template choice: as a runtime branch it
// cost this kernel 8 registers and a CTA per SM).
template <bool SMALL>
__device__ __forceinline__ AdjPair adj_pair(const float4 &pi, const float4 &pj, float dq)
{
    AdjPair p;
    pair_r(pi, pj, p.r, p.rinv, p.dx, p.dy, p.dz);
    const float th = dq * p.r;
    const float th_lo = fmaf(dq, p.r, -th);
    if constexpr (SMALL)
        sincos_small2(0.5f * th, 0.5f * th_lo, p.sh, p.ch);
    else
        sincos_rr2(0.5f * th, 0.5f * th_lo, p.sh, p.ch);
    p.circle = 2.0f * p.ch * p.ch >= 1.0f;
    return p;
}

// sin/cos(q0 r) of a slab seed: exactly (0, 1) at q0 = 0, as sincos_prod gives.
__device__ __forceinline__ void slab_seed(float q0, float r, float &s, float &c)
{
    if (q0 == 0.f) {
        s = 0.f;
        c = 1.f;
    } else {
        sincos_prod(q0, r, s, c);
    }
}

// Sums A (cosine side) and B (sine side) of one pair over all slabs.
__device__ __forceinline__ void adj_pair_sums(const DebyeArgs &a, const float4 *tab,
                                              const float *tab_a, int n_slabs, const AdjPair &p,
                                              float &A, float &B)
{
    float P = 0.f, Q = 0.f;
    for (int sl = 0; sl < n_slabs; ++sl) {
        const int kb = sl * kAdjSlab;
        const int L = (min(kAdjSlab, a.n_q - kb) + 7) & ~7;
        const float4 *t = tab + sl * kAdjStride;
        float s0, c0;
        slab_seed(a.q[kb], p.r, s0, c0);
        if (p.circle) {
            adj_circle_slab(t, L, s0, fmaf(c0, p.ch, s0 * p.sh), 2.0f * p.sh, P, Q);
        } else {
            const float sd = 2.0f * p.sh * p.ch, cd = fmaf(-2.0f * p.sh, p.sh, 1.0f);
            adj_rotate_slab(t, tab_a + sl * kAdjStride, L, s0, c0, sd, cd, P, Q);
        }
    }
    A = p.circle ? P * (0.5f / p.ch) : P;
    B = Q;
}

// Sums of 2 NP pairs, all on the magic-circle form, stepped in NP float2
// lanes (pairs 2v and 2v + 1 share lane v).
template <int NP>
__device__ __forceinline__ void adj_paired_sums(const DebyeArgs &a, const float4 *tab, int n_slabs,
                                                const AdjPair (&p)[2 * NP], float (&A)[2 * NP],
                                                float (&B)[2 * NP])
{
    float2 P[NP], Q[NP], ac[NP];
#pragma unroll
    for (int v = 0; v < NP; ++v) {
        P[v] = make_float2(0.f, 0.f);
        Q[v] = make_float2(0.f, 0.f);
        ac[v] = make_float2(2.0f * p[2 * v].sh, 2.0f * p[2 * v + 1].sh);
    }
    for (int sl = 0; sl < n_slabs; ++sl) {
        const int kb = sl * kAdjSlab;
        const int L = (min(kAdjSlab, a.n_q - kb) + 7) & ~7;
        const float q0 = a.q[kb];
        float2 s[NP], e[NP];
#pragma unroll
        for (int v = 0; v < NP; ++v) {
            float s0, c0, s1, c1;
            const AdjPair &p0 = p[2 * v], &p1 = p[2 * v + 1];
            slab_seed(q0, p0.r, s0, c0);
            slab_seed(q0, p1.r, s1, c1);
            s[v] = make_float2(s0, s1);
            e[v] = make_float2(fmaf(c0, p0.ch, s0 * p0.sh), fmaf(c1, p1.ch, s1 * p1.sh));
        }
        adj_circle_slab_paired<NP>(tab + sl * kAdjStride, L, s, e, ac, P, Q);
    }
#pragma unroll
    for (int v = 0; v < NP; ++v) {
        A[2 * v] = P[v].x * (0.5f / p[2 * v].ch);
        A[2 * v + 1] = P[v].y * (0.5f / p[2 * v + 1].ch);
        B[2 * v] = Q[v].x;
        B[2 * v + 1] = Q[v].y;
    }
}

// Scatters one pair's gradient: the I side into the thread's registers, the J
// side (summed over the warp) into shared memory.
__device__ __forceinline__ void adj_scatter(const AdjPair &p, float A, float B, bool use,
                                            float &gi0, float &gi1, float &gi2, float (*s_gj)[3],
                                            int jj, int lane)
{
    // G = 2 / r^2 * (A - B / r); the J side gets +G*d, the I side -G*d
    float G = 2.0f * p.rinv * p.rinv * fmaf(-B, p.rinv, A);
    G = use ? G : 0.f;
    float gx = G * p.dx, gy = G * p.dy, gz = G * p.dz;
    gi0 -= gx;
    gi1 -= gy;
    gi2 -= gz;
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) {
        gx += __shfl_xor_sync(0xffffffffu, gx, m);
        gy += __shfl_xor_sync(0xffffffffu, gy, m);
        gz += __shfl_xor_sync(0xffffffffu, gz, m);
    }
    if (lane == 0) {
        atomicAdd(&s_gj[jj][0], gx);
        atomicAdd(&s_gj[jj][1], gy);
        atomicAdd(&s_gj[jj][2], gz);
    }
}

// ----------------------------------------------------------------------------
// adjoint through tabulated pair functions (any q grid)
// ----------------------------------------------------------------------------
//
// For one item's type pair (t_i, t_j) the gradient of a pair needs only
//   A(r) = sum_k alpha_k cos(q_k r),   B(r) = sum_k beta_k sin(q_k r)
// (alpha_k = lambda_k f_ti(q_k) f_tj(q_k), beta_k = alpha_k / q_k; q = 0 adds
// nothing to either, since d sinc(q r)/dr vanishes there),
// smooth functions of r alone whose derivatives are bounded by powers of
// q_max.  They are tabulated with their first derivatives on a uniform r grid
// of step h covering every pair distance (adjoint_table_kernel: sums over q in
// FP64), and each pair reads them by cubic Hermite interpolation.  Its error
// is at most h^4 max|f| / 384 with |f| <= q_max^4 sum|alpha|, so below
// (q_max h)^4 / 384 of sum|alpha| (1.6e-8 at q_max h = 0.05, the step the host
// picks) -- smaller than the FP32 recurrence's.  A pair then costs two table
// loads and ~25 FP32 operations instead of 4 per q.
//
// With the implicit water term alpha_k = lambda_k f~_i f~_j is linear in the
// combinations 1, rsasa_i, rsasa_j and rsasa_i rsasa_j, with the factors
// f_ti f_tj, w f_w f_tj, w f_w f_ti and (w f_w)^2: every node then holds four
// entries, one per combination, and a pair weights them with its rsasa.
template <bool WATER>
constexpr int kTableEntries = WATER ? 4 : 1;

// Entry c of node b of the table at r_b = b h (exact in double): A, h dA/dr,
// B, h dB/dr with alpha_k = lambda_k x factor c (c = 0: f_ti f_tj; with water
// 1: w f_w f_tj, 2: w f_w f_ti, 3: (w f_w)^2), by one warp (lane l sums q l,
// l + 32, ...; FP64 partials combined by shuffles; the result is valid in
// every lane).  sin/cos(q r_b) in FP32 with the rounding of q r_b folded in as
// the low part (r_b is carried as hi + lo).
__device__ __forceinline__ float4 adjoint_table_node(const DebyeArgs &a, const float *lambda,
                                                     int ti, int tj, int b, float h, int lane,
                                                     int c = 0)
{
    const double rb = (double)b * (double)h;
    const float r_hi = (float)rb, r_lo = (float)(rb - (double)r_hi);
    double A = 0.0, dA = 0.0, B = 0.0, dB = 0.0;
    for (int k = lane; k < a.n_q; k += 32) {
        const float qk = a.q[k];
        if (qk == 0.f)
            continue; // d sinc(q r) / dr = 0 at q = 0: no term on either side
        const float *row = a.ff + (size_t)k * a.n_types;
        const float fw = c > 0 ? a.water_weight * row[a.water_index] : 0.f;
        const float factor = c == 0   ? row[ti] * row[tj]
                             : c == 1 ? fw * row[tj]
                             : c == 2 ? fw * row[ti]
                                      : fw * fw;
        const float al = lambda[k] * factor;
        const float x = qk * r_hi;
        const float x_lo = fmaf(qk, r_hi, -x) + qk * r_lo;
        float s, c;
        sincos_rr2(x, x_lo, s, c);
        const double be = (double)(al / qk);
        A += (double)al * c;
        dA -= (double)al * qk * s;
        B += be * s;
        dB += be * qk * c;
    }
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) {
        A += __shfl_xor_sync(0xffffffffu, A, m);
        dA += __shfl_xor_sync(0xffffffffu, dA, m);
        B += __shfl_xor_sync(0xffffffffu, B, m);
        dB += __shfl_xor_sync(0xffffffffu, dB, m);
    }
    return make_float4((float)A, (float)(h * dA), (float)B, (float)(h * dB));
}

// A(r) and B(r) of one pair from the table of its item's type pair (nodes of
// kTableEntries<WATER> entries; with water weighted by 1, rs_i, rs_j, rs_i rs_j).
template <bool WATER>
__device__ __forceinline__ void adjoint_table_eval(const float4 *tab, int n_nodes, float h,
                                                   float inv_h, float r, float rs_i, float rs_j,
                                                   float &A, float &B)
{
    constexpr int NT = kTableEntries<WATER>;
    // node index: clamped into the table (a NaN distance reads node 0)
    const float u = fminf(fmaxf(r * inv_h, 0.f), (float)(n_nodes - 2));
    const int b = (int)u;
    const float t = fmaf(-(float)b, h, r) * inv_h; // (r - b h) / h with r - b h rounded once
    const float t2 = t * t, t3 = t2 * t;
    const float h01 = fmaf(-2.0f, t3, 3.0f * t2); // Hermite basis
    const float h00 = 1.0f - h01;
    const float h10 = t3 - 2.0f * t2 + t;
    const float h11 = t3 - t2;
    float m[NT];
    m[0] = 1.0f;
    if (WATER) {
        m[1] = rs_i;
        m[2] = rs_j;
        m[3] = rs_i * rs_j;
    }
    A = 0.f;
    B = 0.f;
#pragma unroll
    for (int c = 0; c < NT; ++c) {
        const float4 p0 = __ldg(tab + (size_t)b * NT + c), p1 = __ldg(tab + (size_t)(b + 1) * NT + c);
        A = fmaf(m[c], fmaf(h00, p0.x, fmaf(h10, p0.y, fmaf(h01, p1.x, h11 * p1.y))), A);
        B = fmaf(m[c], fmaf(h00, p0.z, fmaf(h10, p0.w, fmaf(h01, p1.z, h11 * p1.w))), B);
    }
}

// Adjoint of one work item through the tables: every pair of the item reads
// A and B of its type pair's table, then scatters as the other forms do.  IL
// pairs per step keep IL table loads in flight.
template <int IL, bool WATER = false>
__device__ __forceinline__ void adjoint_table_item(const DebyeArgs &a, int item_idx)
{
    static_assert(3 * IL <= 16, "the J side of a step is reduce-scattered as 16 values");
    constexpr int NT = kTableEntries<WATER>;
    __shared__ float4 s_pos[kBlockAtoms];
    __shared__ float s_rs[WATER ? kBlockAtoms : 1];
    __shared__ float s_gj[kBlockAtoms][3];

    const int tid = threadIdx.x;
    const int lane = tid & 31;
    __syncthreads(); // a previous item of this CTA may still read shared memory
    const PairItem it = a.items[item_idx];
    const BlockDesc bi = a.blocks[it.bi];
    const int tj = a.blocks[it.bj_begin].type;
    const int n_nodes = a.adj_nodes;
    // the item's member (PairItem::pad; 0 for a single structure) owns its tables
    const float4 *tab =
        a.adj_tab +
        ((size_t)it.pad * a.n_types * a.n_types + (size_t)(bi.type * a.n_types + tj)) * n_nodes *
            NT;
    const float h = a.adj_geom ? a.adj_geom[0] : a.adj_h;
    const float inv_h = a.adj_geom ? a.adj_geom[1] : a.adj_inv_h;

    const int i = bi.start + tid;
    const bool valid_i = tid < bi.len;
    const float4 pi = valid_i ? a.pos[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float rs_i = (WATER && valid_i) ? a.rsasa[i] : 0.f;
    float gi0 = 0.f, gi1 = 0.f, gi2 = 0.f;

    for (int b = it.bj_begin; b < it.bj_end; ++b) {
        const BlockDesc bj = a.blocks[b];
        __syncthreads();
        if (tid < bj.len) {
            s_pos[tid] = a.pos[bj.start + tid];
            if (WATER)
                s_rs[tid] = a.rsasa[bj.start + tid];
        }
        s_gj[tid][0] = 0.f;
        s_gj[tid][1] = 0.f;
        s_gj[tid][2] = 0.f;
        __syncthreads();
        const bool diag = (b == it.bi);
        for (int jj = 0; jj < bj.len; jj += IL) {
            AdjPair p[IL] = {};
            float A[IL], B[IL];
#pragma unroll
            for (int v = 0; v < IL; ++v) {
                // past the block's end: a repeated body, masked out below
                const int j = min(jj + v, bj.len - 1);
                pair_r(pi, s_pos[j], p[v].r, p[v].rinv, p[v].dx, p[v].dy, p[v].dz);
                adjoint_table_eval<WATER>(tab, n_nodes, h, inv_h, p[v].r, rs_i,
                                          WATER ? s_rs[j] : 0.f, A[v], B[v]);
            }
            // G d of the step's pairs (zero past the block's end); the I side
            // stays in registers, the J side (IL x 3 values) is reduce-scattered
            // over the warp in one pass and added to shared memory by the lanes
            // that hold the sums
            float w[16];
#pragma unroll
            for (int v = 0; v < IL; ++v) {
                const bool use = jj + v < bj.len && valid_i && (!diag || jj + v > tid);
                float G = 2.0f * p[v].rinv * p[v].rinv * fmaf(-B[v], p[v].rinv, A[v]);
                G = use ? G : 0.f;
                w[3 * v + 0] = G * p[v].dx;
                w[3 * v + 1] = G * p[v].dy;
                w[3 * v + 2] = G * p[v].dz;
                gi0 -= w[3 * v + 0];
                gi1 -= w[3 * v + 1];
                gi2 -= w[3 * v + 2];
            }
#pragma unroll
            for (int k = 3 * IL; k < 16; ++k)
                w[k] = 0.f;
            warp_reduce_scatter<16>(w, lane);
            const int k = lane & 15, v = k / 3;
            if (lane < 16 && k < 3 * IL && jj + v < bj.len)
                atomicAdd(&s_gj[jj + v][k - 3 * v], w[0]);
        }
        __syncthreads();
        if (tid < bj.len) {
            double *g = a.grad + 3 * (size_t)(bj.start + tid);
            atomicAdd(g + 0, (double)s_gj[tid][0]);
            atomicAdd(g + 1, (double)s_gj[tid][1]);
            atomicAdd(g + 2, (double)s_gj[tid][2]);
        }
    }
    if (valid_i) {
        double *g = a.grad + 3 * (size_t)i;
        atomicAdd(g + 0, (double)gi0);
        atomicAdd(g + 1, (double)gi1);
        atomicAdd(g + 2, (double)gi2);
    }
}

// Dynamic shared memory of the adjoint kernels for n_q values.
__host__ __device__ inline size_t adjoint_smem_bytes(int n_q, int qs, bool uniform, bool water)
{
    if (uniform && !water)
        return (size_t)((n_q + kAdjSlab - 1) / kAdjSlab) * kAdjStride *
               (sizeof(float4) + sizeof(float));
    const int n_slabs = (n_q + qs - 1) / qs;
    return (size_t)n_slabs * qs * (water ? 8 : 4) * sizeof(float);
}

// IL pairs per thread step together (8, at 4 CTAs per SM: measured 7 % faster
// than 4 at 7 CTAs per SM, at N = 50,000 and 256 q).
template <int IL, bool SMALL>
__device__ __forceinline__ void adjoint_uniform_item(const DebyeArgs &a, int item_idx)
{
    extern __shared__ float4 s_dyn[];
    __shared__ float4 s_pos[kBlockAtoms];
    __shared__ float s_gj[kBlockAtoms][3];

    const int tid = threadIdx.x;
    const int lane = tid & 31;
    __syncthreads(); // a previous item of this CTA may still read shared memory
    const PairItem it = a.items[item_idx];
    const float *lambda = a.lambda + (size_t)it.pad * a.n_q;
    const BlockDesc bi = a.blocks[it.bi];
    const int tj = a.blocks[it.bj_begin].type;
    const int n_slabs = (a.n_q + kAdjSlab - 1) / kAdjSlab;
    float4 *tab = s_dyn;
    float *tab_a = reinterpret_cast<float *>(s_dyn + n_slabs * kAdjStride);
    adjoint_uniform_table(a, tab, tab_a, n_slabs, lambda, bi.type, tj);

    const int i = bi.start + tid;
    const bool valid_i = tid < bi.len;
    const float4 pi = valid_i ? a.pos[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    float gi0 = 0.f, gi1 = 0.f, gi2 = 0.f;
    const float dq = a.dq;

    for (int b = it.bj_begin; b < it.bj_end; ++b) {
        const BlockDesc bj = a.blocks[b];
        __syncthreads();
        if (tid < bj.len)
            s_pos[tid] = a.pos[bj.start + tid];
        s_gj[tid][0] = 0.f;
        s_gj[tid][1] = 0.f;
        s_gj[tid][2] = 0.f;
        __syncthreads();
        const bool diag = (b == it.bi);
        int jj = 0;
        if (IL > 2) {
            for (; jj + IL - 1 < bj.len; jj += IL) {
                AdjPair p[IL];
                bool all_circle = true;
#pragma unroll
                for (int v = 0; v < IL; ++v) {
                    p[v] = adj_pair<SMALL>(pi, s_pos[jj + v], dq);
                    all_circle = all_circle && p[v].circle;
                }
                float A[IL], B[IL];
                if (all_circle) {
                    adj_paired_sums<IL / 2>(a, tab, n_slabs, p, A, B);
                } else {
#pragma unroll
                    for (int v = 0; v < IL; ++v)
                        adj_pair_sums(a, tab, tab_a, n_slabs, p[v], A[v], B[v]);
                }
#pragma unroll
                for (int v = 0; v < IL; ++v)
                    adj_scatter(p[v], A[v], B[v], valid_i && (!diag || jj + v > tid), gi0, gi1,
                                gi2, s_gj, jj + v, lane);
            }
        }
        for (; jj + 1 < bj.len; jj += 2) {
            const AdjPair p2[2] = {adj_pair<SMALL>(pi, s_pos[jj], dq),
                                   adj_pair<SMALL>(pi, s_pos[jj + 1], dq)};
            float A[2], B[2];
            if (p2[0].circle && p2[1].circle) {
                adj_paired_sums<1>(a, tab, n_slabs, p2, A, B);
            } else {
                adj_pair_sums(a, tab, tab_a, n_slabs, p2[0], A[0], B[0]);
                adj_pair_sums(a, tab, tab_a, n_slabs, p2[1], A[1], B[1]);
            }
            adj_scatter(p2[0], A[0], B[0], valid_i && (!diag || jj > tid), gi0, gi1, gi2, s_gj, jj,
                        lane);
            adj_scatter(p2[1], A[1], B[1], valid_i && (!diag || jj + 1 > tid), gi0, gi1, gi2, s_gj,
                        jj + 1, lane);
        }
        for (; jj < bj.len; ++jj) {
            const AdjPair p = adj_pair<SMALL>(pi, s_pos[jj], dq);
            float A, B;
            adj_pair_sums(a, tab, tab_a, n_slabs, p, A, B);
            adj_scatter(p, A, B, valid_i && (!diag || jj > tid), gi0, gi1, gi2, s_gj, jj, lane);
        }
        __syncthreads();
        if (tid < bj.len) {
            double *g = a.grad + 3 * (size_t)(bj.start + tid);
            atomicAdd(g + 0, (double)s_gj[tid][0]);
            atomicAdd(g + 1, (double)s_gj[tid][1]);
            atomicAdd(g + 2, (double)s_gj[tid][2]);
        }
    }
    if (valid_i) {
        double *g = a.grad + 3 * (size_t)i;
        atomicAdd(g + 0, (double)gi0);
        atomicAdd(g + 1, (double)gi1);
        atomicAdd(g + 2, (double)gi2);
    }
}

// Adjoint of one work item (all q), general form: rotation per pair and
// per-pair water factors, for non-uniform grids and for water.  Adds dL/dx of
// the item's pairs to the FP64 gradient; the item's member (PairItem::pad)
// selects its dL/dI row.
template <int QS, bool UNIFORM, bool WATER>
__device__ __forceinline__ void adjoint_general_item(const DebyeArgs &a, int item_idx, int n_slabs)
{
    extern __shared__ float4 s_dyn[]; // [n_slabs*QS] coefficients (a0, b0, a1, b1)
    __shared__ float4 s_pos[kBlockAtoms];
    __shared__ float s_rs[WATER ? kBlockAtoms : 1];
    __shared__ float s_gj[kBlockAtoms][3];

    const int tid = threadIdx.x;
    const int lane = tid & 31;
    __syncthreads(); // a previous item of this CTA may still read shared memory
    const PairItem it = a.items[item_idx];
    const float *lambda = a.lambda + (size_t)it.pad * a.n_q;
    const BlockDesc bi = a.blocks[it.bi];
    const int tj = a.blocks[it.bj_begin].type;
    const int nqp = n_slabs * QS;
    // per q: alpha = lambda f_i f_j, beta = alpha / q (0 at q == 0); with water
    // the factors are per body, so the table holds lambda, lambda*fw and the
    // type factors, combined per pair below.
    float *coef = reinterpret_cast<float *>(s_dyn);
    for (int k = tid; k < nqp; k += blockDim.x) {
        float l = 0.f, fi = 0.f, fj = 0.f, fw = 0.f, qk = 0.f;
        if (k < a.n_q) {
            l = lambda[k];
            qk = a.q[k];
            fi = a.ff[(size_t)k * a.n_types + bi.type];
            fj = a.ff[(size_t)k * a.n_types + tj];
            fw = WATER ? a.water_weight * a.ff[(size_t)k * a.n_types + a.water_index] : 0.f;
        }
        const float rq = qk != 0.f ? 1.0f / qk : 0.f;
        if (qk == 0.f)
            l = 0.f; // d sinc / dr = 0 at q = 0
        if (WATER) {
            coef[8 * k + 0] = l;
            coef[8 * k + 1] = l * rq;
            coef[8 * k + 2] = fi;
            coef[8 * k + 3] = fj;
            coef[8 * k + 4] = fw;
        } else {
            coef[4 * k + 0] = l * fi * fj;
            coef[4 * k + 1] = l * fi * fj * rq;
        }
    }
    const int i = bi.start + tid;
    const bool valid_i = tid < bi.len;
    const float4 pi = valid_i ? a.pos[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float rs_i = (WATER && valid_i) ? a.rsasa[i] : 0.f;
    float gi0 = 0.f, gi1 = 0.f, gi2 = 0.f;
    const float dq = a.dq;

    for (int b = it.bj_begin; b < it.bj_end; ++b) {
        const BlockDesc bj = a.blocks[b];
        __syncthreads();
        if (tid < bj.len) {
            s_pos[tid] = a.pos[bj.start + tid];
            if (WATER)
                s_rs[tid] = a.rsasa[bj.start + tid];
        }
        s_gj[tid][0] = 0.f;
        s_gj[tid][1] = 0.f;
        s_gj[tid][2] = 0.f;
        __syncthreads();
        const bool diag = (b == it.bi);
        for (int jj = 0; jj < bj.len; ++jj) {
            const float4 pj = s_pos[jj];
            float r, rinv, dx, dy, dz;
            pair_r(pi, pj, r, rinv, dx, dy, dz);
            const bool use = valid_i && (!diag || jj > tid);
            const float rs_j = WATER ? s_rs[jj] : 0.f;
            float A = 0.f, B = 0.f;
            float sd = 0.f, cd = 1.f;
            if (UNIFORM)
                sincos_prod(dq, r, sd, cd);
            for (int sl = 0; sl < n_slabs; ++sl) {
                const int kb = sl * QS;
                if (UNIFORM) {
                    float s, c;
                    sincos_prod(a.q[min(kb, a.n_q - 1)], r, s, c);
#pragma unroll
                    for (int k = 0; k < QS; ++k) {
                        float al, be;
                        if (WATER) {
                            const float *cf = coef + 8 * (kb + k);
                            const float f1 = fmaf(rs_i, cf[4], cf[2]);
                            const float f2 = fmaf(rs_j, cf[4], cf[3]);
                            const float ff = f1 * f2;
                            al = cf[0] * ff;
                            be = cf[1] * ff;
                        } else {
                            const float2 ab = *reinterpret_cast<const float2 *>(coef + 4 * (kb + k));
                            al = ab.x;
                            be = ab.y;
                        }
                        A = fmaf(al, c, A);
                        B = fmaf(be, s, B);
                        const float sn = fmaf(c, sd, s * cd);
                        const float cn = fmaf(-s, sd, c * cd);
                        s = sn;
                        c = cn;
                    }
                } else {
#pragma unroll 4
                    for (int k = 0; k < QS; ++k) {
                        const int kk = kb + k;
                        if (kk >= a.n_q)
                            break;
                        float s, c;
                        sincos_prod(a.q[kk], r, s, c);
                        float al, be;
                        if (WATER) {
                            const float *cf = coef + 8 * kk;
                            const float ff = fmaf(rs_i, cf[4], cf[2]) * fmaf(rs_j, cf[4], cf[3]);
                            al = cf[0] * ff;
                            be = cf[1] * ff;
                        } else {
                            al = coef[4 * kk + 0];
                            be = coef[4 * kk + 1];
                        }
                        A = fmaf(al, c, A);
                        B = fmaf(be, s, B);
                    }
                }
            }
            // G = 2 / r^2 * (A - B / r); the J side gets +G*d, the I side -G*d
            float G = 2.0f * rinv * rinv * fmaf(-B, rinv, A);
            G = use ? G : 0.f;
            float gx = G * dx, gy = G * dy, gz = G * dz;
            gi0 -= gx;
            gi1 -= gy;
            gi2 -= gz;
#pragma unroll
            for (int m = 16; m >= 1; m >>= 1) {
                gx += __shfl_xor_sync(0xffffffffu, gx, m);
                gy += __shfl_xor_sync(0xffffffffu, gy, m);
                gz += __shfl_xor_sync(0xffffffffu, gz, m);
            }
            if (lane == 0) {
                atomicAdd(&s_gj[jj][0], gx);
                atomicAdd(&s_gj[jj][1], gy);
                atomicAdd(&s_gj[jj][2], gz);
            }
        }
        __syncthreads();
        if (tid < bj.len) {
            double *g = a.grad + 3 * (size_t)(bj.start + tid);
            atomicAdd(g + 0, (double)s_gj[tid][0]);
            atomicAdd(g + 1, (double)s_gj[tid][1]);
            atomicAdd(g + 2, (double)s_gj[tid][2]);
        }
    }
    if (valid_i) {
        double *g = a.grad + 3 * (size_t)i;
        atomicAdd(g + 0, (double)gi0);
        atomicAdd(g + 1, (double)gi1);
        atomicAdd(g + 2, (double)gi2);
    }
}

template <int QS, bool UNIFORM, bool WATER, bool SMALL = false>
__device__ __forceinline__ void adjoint_item(const DebyeArgs &a, int item_idx, int n_slabs)
{
    if constexpr (UNIFORM && !WATER)
        adjoint_uniform_item<8, SMALL>(a, item_idx);
    else
        adjoint_general_item<QS, UNIFORM, WATER>(a, item_idx, n_slabs);
}

// ----------------------------------------------------------------------------
// forward, uniform q grid without water: chained slabs
// ----------------------------------------------------------------------------
//
// A work item over a chain of up to two 192-q slabs and a QT-q tail: the J
// side is taken kChainPairs bodies at a time; every pair chain of such a
// sub-tile is seeded once, at the start of the chain, runs through the first
// slab, leaves its recurrence state (s, d of the even/odd sequences, lam with
// the sign of the odd steps) in shared memory while the slab's sums are
// reduce-scattered into per-lane FP64 accumulators (shared memory: lane L
// owns q index 32 c + L of every slab), and resumes from it in the next slab.

template <int QS, int QH, bool SIGNED>
__device__ __forceinline__ void chain_steps(WideSeed &p1, WideSeed &p2, float2 (&S)[QH])
{
    if constexpr (SIGNED) {
        if (__any_sync(0xffffffffu, p1.sg < 0.f || p2.sg < 0.f))
            wide_pair2_carry<QS, QH, true>(p1, p2, S);
        else
            wide_pair2_carry<QS, QH, false>(p1, p2, S);
    } else {
        wide_pair2_carry<QS, QH, false>(p1, p2, S);
    }
}

// Forward pair sums of one work item over the chain q [k0, k0 + chain_q)
// (n_main 192-q slabs, then a QT-q tail): writes partial[k][item_idx] = sum
// over the item's pairs of f_i f_j sin(q_k r)/r.  q_slots = n_main * 192 + QT
// rounded up to 32 (the accumulator stride); dsm: chain_smem_bytes(q_slots)
// of dynamic shared memory.  Called once per CTA by forward_chain_kernel and
// repeatedly by the persistent batch kernel (hence the leading barrier).
// X0_FIRST: the seeds of wide_seed_x0_first.
template <int QT, bool SIGNED, bool X0_FIRST = false>
__device__ __forceinline__ void forward_chain_item(const DebyeArgs &a, int item_idx, int k0,
                                                   int chain_q, int n_main, int q_slots,
                                                   unsigned char *dsm)
{
    constexpr int QM = kChainMain, QH = QM / 2, T = kChainPairs;
    static_assert(QT % 8 == 0 && QT <= QM, "tail slab");
    __shared__ float4 s_pos[kBlockAtoms];
    float2 *st_sd = reinterpret_cast<float2 *>(dsm);                       // [T][2][128]
    float *st_l = reinterpret_cast<float *>(dsm + sizeof(float2) * 2 * T * kBlockAtoms); // [T][128]
    double *acc = reinterpret_cast<double *>(dsm + chain_state_bytes());   // [4][q_slots]

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    __syncthreads(); // a previous item of this CTA may still read shared memory
    const PairItem it = a.items[item_idx];
    const BlockDesc bi = a.blocks[it.bi];
    const int tj = a.blocks[it.bj_begin].type;
    const int i = bi.start + tid;
    const bool valid_i = tid < bi.len;
    const float4 pi = valid_i ? a.pos[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float q0 = a.q[k0];
    const float dq = a.dq;
    const bool small_th = !SIGNED || a.small_theta >= 2;
    const int n_slabs = n_main + (QT > 0 ? 1 : 0);

    double *my_acc = acc + (size_t)warp * q_slots;
    for (int k = lane; k < q_slots; k += 32)
        my_acc[k] = 0.0;

    for (int b = it.bj_begin; b < it.bj_end; ++b) {
        const BlockDesc bj = a.blocks[b];
        __syncthreads();
        // slots past the block's end repeat its last body: a finite pair
        // distance, and the pair is masked
        s_pos[tid] = a.pos[bj.start + min(tid, bj.len - 1)];
        __syncthreads();
        const bool diag = (b == it.bi);
        for (int sub = 0; sub < bj.len; sub += T) {
            const int np = min(T, bj.len - sub);
            for (int s = 0; s < n_slabs; ++s) {
                const bool first = s == 0, last = s == n_slabs - 1, tail = s >= n_main;
                float2 S[QH];
#pragma unroll
                for (int m = 0; m < QH; ++m)
                    S[m] = make_float2(0.f, 0.f);
                for (int jp = 0; jp < np; jp += 2) {
                    const int j = sub + jp;
                    WideSeed p1, p2;
                    float2 *sd = st_sd + (size_t)jp * 2 * kBlockAtoms + tid;
                    float *sl = st_l + (size_t)jp * kBlockAtoms + tid;
                    if (first) {
                        float r1, ri1, r2, ri2, dx, dy, dz;
                        pair_r(pi, s_pos[j], r1, ri1, dx, dy, dz);
                        pair_r(pi, s_pos[min(j + 1, kBlockAtoms - 1)], r2, ri2, dx, dy, dz);
                        const bool u1 = valid_i && (!diag || j > tid);
                        const bool u2 = valid_i && jp + 1 < np && (!diag || j + 1 > tid);
                        if constexpr (X0_FIRST) {
                            p1 = wide_seed_x0_first(q0, dq, r1, u1 ? ri1 : 0.f, small_th);
                            p2 = wide_seed_x0_first(q0, dq, r2, u2 ? ri2 : 0.f, small_th);
                        } else {
                            p1 = wide_seed(q0, dq, r1, u1 ? ri1 : 0.f, small_th);
                            p2 = wide_seed(q0, dq, r2, u2 ? ri2 : 0.f, small_th);
                        }
                    } else {
                        p1.s = sd[0];
                        p1.d = sd[kBlockAtoms];
                        p2.s = sd[2 * kBlockAtoms];
                        p2.d = sd[3 * kBlockAtoms];
                        unpack_lam_sign(sl[0], p1.l, p1.sg);
                        unpack_lam_sign(sl[kBlockAtoms], p2.l, p2.sg);
                    }
                    if (tail) {
                        if constexpr (QT > 0)
                            chain_steps<QT, QH, SIGNED>(p1, p2, S);
                    } else {
                        chain_steps<QM, QH, SIGNED>(p1, p2, S);
                    }
                    if (!last) {
                        sd[0] = p1.s;
                        sd[kBlockAtoms] = p1.d;
                        sd[2 * kBlockAtoms] = p2.s;
                        sd[3 * kBlockAtoms] = p2.d;
                        sl[0] = pack_lam_sign(p1.l, p1.sg);
                        sl[kBlockAtoms] = pack_lam_sign(p2.l, p2.sg);
                    }
                }
                // the slab's sums of this sub-tile into the lane accumulators
                const int base = s * QM;
                const int n_chunks = tail ? (QT + 31) / 32 : QM / 32;
#pragma unroll
                for (int c = 0; c < QM / 32; ++c) {
                    if (c >= n_chunks)
                        break;
                    float v[32];
#pragma unroll
                    for (int k = 0; k < 32; ++k)
                        v[k] = pair_at(S, 32 * c + k);
                    warp_reduce_scatter<32>(v, lane);
                    my_acc[base + 32 * c + lane] += (double)v[0];
                }
            }
        }
    }
    __syncthreads();
    for (int k = tid; k < chain_q; k += kBlockAtoms) {
        const int kk = k0 + k;
        if (kk >= a.n_q)
            continue;
        double s = 0.0;
#pragma unroll
        for (int w = 0; w < kBlockAtoms / 32; ++w)
            s += acc[(size_t)w * q_slots + k];
        const double fi = a.ff[(size_t)kk * a.n_types + bi.type];
        const double fj = a.ff[(size_t)kk * a.n_types + tj];
        a.partial[(size_t)kk * a.n_items + item_idx] = s * fi * fj;
    }
}

} // namespace rsx
