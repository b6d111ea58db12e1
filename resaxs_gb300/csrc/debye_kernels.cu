// Debye pair kernels for sm_103a: forward I(q), incremental delta I(q) and
// the adjoint dL/dx.  Written from scratch for this project.
//
// Common structure
//  * Bodies are stored in type-sorted order and cut into block tiles of at
//    most 128 bodies of one type (BlockDesc), so every (I-block, J-block) pair
//    of tiles has a single pair of form factors F[q][t_i] * F[q][t_j].
//  * One CTA of 128 threads owns an I-block (one body per thread) and streams
//    its J-blocks through shared memory with one float4 load per thread.
//  * A CTA covers a slab of QS consecutive q values.  On a uniform q grid the
//    per-pair values sin(q_k r)/r, cos(q_k r)/r for the slab are produced by
//    rotating the pair (s, c) by the angle dq*r: 4 FP32 ops per q instead of a
//    sine evaluation.  The seeds sin/cos(q_0 r) and sin/cos(dq r) come from an
//    explicit Cody-Waite range reduction plus the Taylor series (rsx_math.cuh),
//    so they carry relative accuracy even for tiny arguments, and the rotation
//    keeps that relative accuracy (error grows ~ k*eps over the slab).
//    sinc(q r) = (sin(q r)/r) / q: the 1/q factor is applied once per q in FP64
//    when the curve is assembled.
//  * Per-thread sums: plain FP32 over one J-block, then folded into a Kahan
//    (compensated) accumulator per q.  Warp-level: a reduce-scatter with
//    shuffles (lane k ends with q index k).  Across warps and CTAs: FP64.
#include "rsx_internal.h"
#include "rsx_math.cuh"

#include <atomic>

namespace rsx {

static std::atomic<unsigned long long> g_launches{0};
void count_launch(int n) { g_launches += (unsigned long long)n; }
unsigned long long launch_count() { return g_launches.load(); }

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
// then give sinc = 1, as the reference's device kernel does).
__device__ __forceinline__ void pair_r(const float4 &a, const float4 &b, float &r, float &rinv,
                                       float &dx, float &dy, float &dz)
{
    dx = b.x - a.x;
    dy = b.y - a.y;
    dz = b.z - a.z;
    float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
    r2 = fmaxf(r2, 1e-12f);
    rinv = rsqrtf(r2);
    r = r2 * rinv;
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

__device__ __forceinline__ PairSeed pair_seed(float x0, float th, float sc)
{
    PairSeed p;
    float s0, c0, sh, ch;
    sincos_rr(x0, s0, c0);
    sincos_any(0.5f * th, sh, ch);
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

template <int QS, bool UNIFORM, bool WATER>
__global__ void __launch_bounds__(kBlockAtoms) forward_kernel(const DebyeArgs a)
{
    __shared__ float4 s_pos[kBlockAtoms];
    __shared__ float s_rs[WATER ? kBlockAtoms : 1];
    __shared__ float s_q[QS], s_fi[QS], s_fj[QS], s_fw[QS];
    __shared__ float s_comp[QS][kBlockAtoms];                 // Kahan terms, per thread
    __shared__ float s_compw[WATER ? QS : 1][kBlockAtoms];
    __shared__ double s_red[kBlockAtoms / 32][QS];

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const PairItem it = a.items[blockIdx.x];
    const BlockDesc bi = a.blocks[it.bi];
    const int tj = a.blocks[it.bj_begin].type;
    const int k0 = a.k_base + blockIdx.y * QS;
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
                const PairSeed p1 = pair_seed(q0 * r1, dq * r1, u1 ? ri1 : 0.f);
                const PairSeed p2 = pair_seed(q0 * r2, dq * r2, u2 ? ri2 : 0.f);
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
                const PairSeed p = pair_seed(q0 * r, dq * r, sc);
                pair_slab<QS, WATER>(p, rs_j, S, SW);
            } else {
#pragma unroll
                for (int k = 0; k < QS; ++k) {
                    float sk, ck;
                    sincos_rr(s_q[k] * r, sk, ck);
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
        a.partial[(size_t)(k0 + k) * a.n_items + blockIdx.x] = s;
    }
}

// ----------------------------------------------------------------------------
// assemble I(q) = self(q) + 2 * cross(q) / q  (q = 0: (sum f)^2)
// ----------------------------------------------------------------------------

__global__ void __launch_bounds__(256) assemble_kernel(const AssembleArgs a)
{
    __shared__ double s_w[8];
    const int k = blockIdx.x;
    double s = 0.0;
    const double *row = a.partial + (size_t)k * a.n_parts;
    for (int x = threadIdx.x; x < a.n_parts; x += blockDim.x)
        s += row[x];
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1)
        s += __shfl_xor_sync(0xffffffffu, s, m);
    if ((threadIdx.x & 31) == 0)
        s_w[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x != 0)
        return;
    double cross = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w)
        cross += s_w[w];
    const double q = a.q[k];
    if (a.accumulate) {
        if (q != 0.0)
            a.iq64[k] += 2.0 * cross / q;
    } else {
        double self = 0.0, sumf = 0.0;
        const float *row_ff = a.ff + (size_t)k * a.n_types;
        const double fw = a.has_water ? (double)(a.water_weight * row_ff[a.water_index]) : 0.0;
        for (int t = 0; t < a.n_types; ++t) {
            const double F = row_ff[t];
            self += a.type_count[t] * F * F;
            sumf += a.type_count[t] * F;
            if (a.has_water)
                self += 2.0 * fw * F * a.rsasa_sum[t];
        }
        if (a.has_water) {
            self += fw * fw * a.rsasa_sq_sum;
            sumf += fw * a.rsasa_total;
        }
        a.iq64[k] = (q != 0.0) ? self + 2.0 * cross / q : sumf * sumf;
    }
    a.iq32[k] = (float)a.iq64[k];
}

// ----------------------------------------------------------------------------
// incremental: delta of the cross sum when the moved list changes position
// ----------------------------------------------------------------------------

template <int QS, bool UNIFORM>
__global__ void __launch_bounds__(kBlockAtoms) delta_kernel(const DeltaArgs a)
{
    __shared__ float4 s_new[kBlockAtoms], s_old[kBlockAtoms];
    __shared__ int s_idx[kBlockAtoms];
    __shared__ float s_q[QS], s_fy[QS], s_fx[QS];
    __shared__ double s_red[kBlockAtoms / 32][QS];

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const BlockDesc by = a.blocks[blockIdx.x];
    const int k0 = blockIdx.y * QS;
    if (tid < QS) {
        const int k = k0 + tid;
        const bool in = k < a.n_q;
        s_q[tid] = in ? a.q[k] : 0.f;
        s_fy[tid] = in ? a.ff[(size_t)k * a.n_types + by.type] : 0.f;
    }
    const int y = by.start + tid;
    const bool valid = tid < by.len;
    const float4 py_old = valid ? a.pos_old[y] : make_float4(0.f, 0.f, 0.f, 0.f);
    const int slot = valid ? a.moved_slot[y] : -1;
    const float4 py_new = slot >= 0 ? a.moved_new[slot] : py_old;
    // pairs with a static body are met once (weight 1); pairs inside the moved
    // list are met from both ends (weight 1/2 each)
    const float mult = slot >= 0 ? 0.5f : 1.0f;

    float acc[QS], comp[QS];
#pragma unroll
    for (int k = 0; k < QS; ++k) {
        acc[k] = 0.f;
        comp[k] = 0.f;
    }
    const float dq = a.dq;
    for (int mt = 0; mt < a.n_mtiles; ++mt) {
        const BlockDesc tile = a.mtiles[mt];
        __syncthreads();
        if (tid < tile.len) {
            const int m = tile.start + tid;
            const int idx = a.moved_idx[m];
            s_new[tid] = a.moved_new[m];
            s_old[tid] = a.pos_old[idx];
            s_idx[tid] = idx;
        }
        if (tid < QS)
            s_fx[tid] = (k0 + tid < a.n_q) ? a.ff[(size_t)(k0 + tid) * a.n_types + tile.type] : 0.f;
        __syncthreads();
        const float q0 = s_q[0];
        float S[QS];
#pragma unroll
        for (int k = 0; k < QS; ++k)
            S[k] = 0.f;
        for (int jj = 0; jj < tile.len; ++jj) {
            const bool use = valid && s_idx[jj] != y;
            float rn, rninv, ro, roinv, dx, dy, dz;
            pair_r(py_new, s_new[jj], rn, rninv, dx, dy, dz);
            pair_r(py_old, s_old[jj], ro, roinv, dx, dy, dz);
            const float scn = use ? rninv : 0.f;
            const float sco = use ? roinv : 0.f;
            if (UNIFORM) {
                float sn0, cn0, sdn, cdn, so0, co0, sdo, cdo;
                sincos_rr(q0 * rn, sn0, cn0);
                sincos_any(dq * rn, sdn, cdn);
                sincos_rr(q0 * ro, so0, co0);
                sincos_any(dq * ro, sdo, cdo);
                float sn = sn0 * scn, cn = cn0 * scn, so = so0 * sco, co = co0 * sco;
#pragma unroll
                for (int k = 0; k < QS; ++k) {
                    S[k] += sn - so;
                    const float sn2 = fmaf(cn, sdn, sn * cdn);
                    const float cn2 = fmaf(-sn, sdn, cn * cdn);
                    const float so2 = fmaf(co, sdo, so * cdo);
                    const float co2 = fmaf(-so, sdo, co * cdo);
                    sn = sn2;
                    cn = cn2;
                    so = so2;
                    co = co2;
                }
            } else {
#pragma unroll
                for (int k = 0; k < QS; ++k) {
                    float s1, c1, s2, c2;
                    sincos_rr(s_q[k] * rn, s1, c1);
                    sincos_rr(s_q[k] * ro, s2, c2);
                    S[k] += s1 * scn - s2 * sco;
                }
            }
        }
#pragma unroll
        for (int k = 0; k < QS; ++k)
            kahan_add(acc[k], comp[k], s_fx[k] * S[k]);
    }
    float v[QS];
#pragma unroll
    for (int k = 0; k < QS; ++k)
        v[k] = valid ? mult * (acc[k] - comp[k]) : 0.f;
    warp_reduce_scatter<QS>(v, lane);
    if (lane < QS)
        s_red[warp][lane] = (double)v[0];
    __syncthreads();
    if (tid < QS && k0 + tid < a.n_q) {
        double s = 0.0;
#pragma unroll
        for (int w = 0; w < kBlockAtoms / 32; ++w)
            s += s_red[w][tid];
        a.partial[(size_t)(k0 + tid) * a.n_blocks + blockIdx.x] = s * (double)s_fy[tid];
    }
}

__global__ void apply_moves_kernel(float4 *pos, const float4 *moved_new, const int *moved_idx,
                                   int k)
{
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m < k)
        pos[moved_idx[m]] = moved_new[m];
}

// slot[idx[m]] = m (set) or -1 (clear) for the moved list
__global__ void mark_moved_kernel(int *slot, const int *moved_idx, int k, int set)
{
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m < k)
        slot[moved_idx[m]] = set ? m : -1;
}

__global__ void f64_to_f32_kernel(const double *src, float *dst, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        dst[i] = (float)src[i];
}

// ----------------------------------------------------------------------------
// adjoint: grad_i = sum_j G_ij (x_i - x_j),
//   G_ij = 2/r^2 sum_q lambda_q f_i f_j (cos(q r) - sinc(q r))
// Each pair is visited once (upper triangle); the J side of every pair is
// summed over the warp with shuffles, accumulated in shared memory and
// flushed to the FP64 gradient once per J-block.  The thread runs the whole
// q range for each pair (slab by slab, all in registers), so the gradient of
// a pair is complete before it is scattered.
// ----------------------------------------------------------------------------

template <int QS, bool UNIFORM, bool WATER>
__global__ void __launch_bounds__(kBlockAtoms) adjoint_kernel(const DebyeArgs a, int n_slabs)
{
    extern __shared__ float4 s_dyn[]; // [n_slabs*QS] coefficients (a0, b0, a1, b1)
    __shared__ float4 s_pos[kBlockAtoms];
    __shared__ float s_rs[WATER ? kBlockAtoms : 1];
    __shared__ float s_gj[kBlockAtoms][3];

    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const PairItem it = a.items[blockIdx.x];
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
            l = a.lambda[k];
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
                sincos_any(dq * r, sd, cd);
            for (int sl = 0; sl < n_slabs; ++sl) {
                const int kb = sl * QS;
                if (UNIFORM) {
                    float s, c;
                    sincos_rr(a.q[min(kb, a.n_q - 1)] * r, s, c);
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
                        sincos_rr(a.q[kk] * r, s, c);
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

// ----------------------------------------------------------------------------
// launchers
// ----------------------------------------------------------------------------

template <int QS, bool U, bool W>
static cudaError_t forward_launch(DebyeArgs a, int k_base, int n_slabs, cudaStream_t st)
{
    a.k_base = k_base;
    const dim3 grid(a.n_items, n_slabs);
    forward_kernel<QS, U, W><<<grid, kBlockAtoms, 0, st>>>(a);
    count_launch();
    return cudaGetLastError();
}

template <int QS>
static cudaError_t forward_qs(const DebyeArgs &a, int k_base, int n_slabs, bool uniform,
                              bool water, cudaStream_t st)
{
    if (uniform && !water)
        return forward_launch<QS, true, false>(a, k_base, n_slabs, st);
    if (uniform && water)
        return forward_launch<QS, true, true>(a, k_base, n_slabs, st);
    if (!uniform && !water)
        return forward_launch<QS, false, false>(a, k_base, n_slabs, st);
    return forward_launch<QS, false, true>(a, k_base, n_slabs, st);
}

static cudaError_t forward_dispatch(const DebyeArgs &a, int qs, int k_base, int n_slabs,
                                    bool uniform, bool water, cudaStream_t st)
{
    switch (qs) {
    case 8:
        return forward_qs<8>(a, k_base, n_slabs, uniform, water, st);
    case 16:
        return forward_qs<16>(a, k_base, n_slabs, uniform, water, st);
    case 32:
        return forward_qs<32>(a, k_base, n_slabs, uniform, water, st);
    case 64: // uniform grid without water only (register budget)
        return (uniform && !water) ? forward_launch<64, true, false>(a, k_base, n_slabs, st)
                                   : cudaErrorInvalidValue;
    default:
        return cudaErrorInvalidValue;
    }
}

// Full slabs of q_slab values, then the remainder in the smallest slab of
// 8 / 16 / 32 that covers it (a second launch on the same stream).
cudaError_t launch_forward(const DebyeArgs &a, int q_slab, bool uniform, bool water,
                           cudaStream_t st)
{
    if (a.n_items == 0)
        return cudaSuccess;
    const int full = a.n_q / q_slab;
    const int rest = a.n_q - full * q_slab;
    if (full > 0) {
        cudaError_t e = forward_dispatch(a, q_slab, 0, full, uniform, water, st);
        if (e != cudaSuccess)
            return e;
    }
    if (rest > 0) {
        const int tail = rest <= 8 ? 8 : (rest <= 16 ? 16 : (rest <= 32 ? 32 : q_slab));
        const int n_tail = (rest + tail - 1) / tail;
        return forward_dispatch(a, tail, full * q_slab, n_tail, uniform, water, st);
    }
    return cudaSuccess;
}

cudaError_t launch_assemble(const AssembleArgs &a, cudaStream_t st)
{
    assemble_kernel<<<a.n_q, 256, 0, st>>>(a);
    count_launch();
    return cudaGetLastError();
}

template <int QS>
static cudaError_t delta_qs(const DeltaArgs &a, bool uniform, cudaStream_t st)
{
    const dim3 grid(a.n_blocks, (a.n_q + QS - 1) / QS);
    if (uniform)
        delta_kernel<QS, true><<<grid, kBlockAtoms, 0, st>>>(a);
    else
        delta_kernel<QS, false><<<grid, kBlockAtoms, 0, st>>>(a);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_delta(const DeltaArgs &a, int q_slab, bool uniform, cudaStream_t st)
{
    if (a.n_blocks == 0 || a.k == 0)
        return cudaSuccess;
    switch (q_slab) {
    case 8:
        return delta_qs<8>(a, uniform, st);
    case 16:
        return delta_qs<16>(a, uniform, st);
    case 32:
        return delta_qs<32>(a, uniform, st);
    default:
        return cudaErrorInvalidValue;
    }
}

cudaError_t launch_apply_moves(float4 *pos, const float4 *moved_new, const int *moved_idx,
                               int k, cudaStream_t st)
{
    if (k == 0)
        return cudaSuccess;
    apply_moves_kernel<<<(k + 255) / 256, 256, 0, st>>>(pos, moved_new, moved_idx, k);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_mark_moved(int *slot, const int *moved_idx, int k, int set, cudaStream_t st)
{
    if (k == 0)
        return cudaSuccess;
    mark_moved_kernel<<<(k + 255) / 256, 256, 0, st>>>(slot, moved_idx, k, set);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_f64_to_f32(const double *src, float *dst, int n, cudaStream_t st)
{
    if (n == 0)
        return cudaSuccess;
    f64_to_f32_kernel<<<(n + 255) / 256, 256, 0, st>>>(src, dst, n);
    count_launch();
    return cudaGetLastError();
}

template <int QS>
static cudaError_t adjoint_qs(const DebyeArgs &a, bool uniform, bool water, cudaStream_t st)
{
    const int n_slabs = (a.n_q + QS - 1) / QS;
    const size_t smem = (size_t)n_slabs * QS * (water ? 8 : 4) * sizeof(float);
    const dim3 grid(a.n_items);
    cudaError_t e = cudaSuccess;
#define RSX_ADJ(U, W)                                                                      \
    do {                                                                                   \
        auto kfn = adjoint_kernel<QS, U, W>;                                               \
        if (smem > 48 * 1024)                                                              \
            e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize,     \
                                     (int)smem);                                           \
        if (e == cudaSuccess)                                                              \
            kfn<<<grid, kBlockAtoms, smem, st>>>(a, n_slabs);                              \
    } while (0)
    if (uniform && !water)
        RSX_ADJ(true, false);
    else if (uniform && water)
        RSX_ADJ(true, true);
    else if (!uniform && !water)
        RSX_ADJ(false, false);
    else
        RSX_ADJ(false, true);
#undef RSX_ADJ
    if (e != cudaSuccess)
        return e;
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_adjoint(const DebyeArgs &a, int q_slab, bool uniform, bool water,
                           cudaStream_t st)
{
    if (a.n_items == 0)
        return cudaSuccess;
    switch (q_slab) {
    case 8:
        return adjoint_qs<8>(a, uniform, water, st);
    case 16:
        return adjoint_qs<16>(a, uniform, water, st);
    case 32:
        return adjoint_qs<32>(a, uniform, water, st);
    default:
        return cudaErrorInvalidValue;
    }
}

} // namespace rsx
