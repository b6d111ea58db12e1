// Device-side building blocks of the Debye pair kernels, shared by the
// per-structure launches (debye_kernels.cu) and the persistent batch kernels
// (batch_kernels.cu).  Written from scratch for this project; see
// debye_kernels.cu for the overall scheme.
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

__device__ __forceinline__ void kahan_add(float &acc, float &comp, float x)
{
    const float y = x - comp;
    const float t = acc + y;
    comp = (t - acc) - y;
    acc = t;
}

// Distance terms of one pair: r and 1/r with r >= 1e-6 (coincident bodies
// then give sinc = 1, as the reference's device kernel does).  Both are
// correctly rounded (IEEE sqrt and division): the hardware reciprocal square
// root approximation has a systematic error that, over 1e10 pairs, shifts
// I(q) at high q by ~1e-4 relative (measured against the FP64 oracle at
// 50,000 and 200,000 bodies); the rounded forms cost ~10% of the forward.
__device__ __forceinline__ void pair_r(const float4 &a, const float4 &b, float &r, float &rinv,
                                       float &dx, float &dy, float &dz)
{
    dx = b.x - a.x;
    dy = b.y - a.y;
    dz = b.z - a.z;
    float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
    r2 = fmaxf(r2, 1e-12f);
    r = __fsqrt_rn(r2);
    rinv = __frcp_rn(r);
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

// Adjoint of one work item (all q): adds dL/dx of the item's pairs to the
// FP64 gradient.  The item's member (PairItem::pad) selects its dL/dI row.
template <int QS, bool UNIFORM, bool WATER>
__device__ __forceinline__ void adjoint_item(const DebyeArgs &a, int item_idx, int n_slabs)
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

} // namespace rsx
