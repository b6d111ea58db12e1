// Forward on q grids without the uniform-step recurrence (non-uniform grids,
// no water) through the gridded pair-distance distribution.  Written from
// scratch for this project.
//
// For one type pair the cross sum needs sum_p g_q(r_p), g_q(r) = sin(q r)/r,
// for every q.  Each pair deposits its cubic Hermite weights onto the two
// nodes around its distance on a uniform r grid of step h: value weights W
// (h00, h01) and derivative weights D (h10, h11).  Then
//     sum_p g_q(r_p) ~= sum_b W_b g_q(r_b) + D_b h g_q'(r_b)
// is evaluated per q over the nodes.  This is the transpose of reading g_q at
// every pair by Hermite interpolation, so the error per pair is the
// interpolation error: g_q = q j0(q r) has |g''''| <= q^5 / 5, which bounds it
// by (q h)^4 / 1920 of q (3.3e-9 at q_max h = 0.05, the step the host picks).
// The work per pair no longer depends on Q: a distance, four weights and four
// shared-memory atomic adds.
//
// A work item's histograms are accumulated in shared memory in 64-bit fixed
// point (units of 2^-32): integer adds are exact in any order, and a node can
// take 2^31 unit weights from one item before the sum could overflow (an
// item has at most 128 x n bodies' pairs).  A weight is quantised to 2^-32
// (2.3e-10).  The items' sums are then added into FP64 global histograms
// (relative rounding ~1e-16 per add).
#include "debye_device.cuh"

namespace rsx {

constexpr double kGridUnit = 4294967296.0; // 2^32

__device__ __forceinline__ unsigned long long grid_fixed(float w)
{
    return (unsigned long long)__double2ll_rn((double)w * kGridUnit);
}

// One CTA per forward work item (one type pair): the item's pairs deposit into
// shared-memory histograms [2][nodes] (W then D), which are then added to the
// type pair's FP64 global histograms.
__global__ void __launch_bounds__(kBlockAtoms)
    forward_grid_deposit_kernel(const DebyeArgs a, double *hist, int nodes, float h, float inv_h)
{
    extern __shared__ unsigned long long s_hist[]; // [2 * nodes]
    __shared__ float4 s_pos[kBlockAtoms];
    const int tid = threadIdx.x;
    for (int k = tid; k < 2 * nodes; k += kBlockAtoms)
        s_hist[k] = 0ull;
    const PairItem it = a.items[blockIdx.x];
    const BlockDesc bi = a.blocks[it.bi];
    const int tj = a.blocks[it.bj_begin].type;
    const int i = bi.start + tid;
    const bool valid_i = tid < bi.len;
    const float4 pi = valid_i ? a.pos[i] : make_float4(0.f, 0.f, 0.f, 0.f);

    for (int b = it.bj_begin; b < it.bj_end; ++b) {
        const BlockDesc bj = a.blocks[b];
        __syncthreads(); // also orders the histogram clearing before the first adds
        if (tid < bj.len)
            s_pos[tid] = a.pos[bj.start + tid];
        __syncthreads();
        const bool diag = (b == it.bi);
        if (!valid_i)
            continue;
        for (int jj = diag ? tid + 1 : 0; jj < bj.len; ++jj) {
            float r, ri, dx, dy, dz;
            pair_r(pi, s_pos[jj], r, ri, dx, dy, dz);
            // node index clamped into the grid (a NaN distance goes to node 0)
            const float u = fminf(fmaxf(r * inv_h, 0.f), (float)(nodes - 2));
            const int n = (int)u;
            const float t = fmaf(-(float)n, h, r) * inv_h;
            const float t2 = t * t, t3 = t2 * t;
            const float h01 = fmaf(-2.0f, t3, 3.0f * t2);
            const float h00 = 1.0f - h01;
            const float h10 = t3 - 2.0f * t2 + t;
            const float h11 = t3 - t2;
            atomicAdd(&s_hist[n], grid_fixed(h00));
            atomicAdd(&s_hist[n + 1], grid_fixed(h01));
            atomicAdd(&s_hist[nodes + n], grid_fixed(h10));
            atomicAdd(&s_hist[nodes + n + 1], grid_fixed(h11));
        }
    }
    __syncthreads();
    double *dst = hist + (size_t)(bi.type * a.n_types + tj) * 2 * nodes;
    for (int k = tid; k < 2 * nodes; k += kBlockAtoms) {
        const long long v = (long long)s_hist[k];
        if (v != 0)
            atomicAdd(dst + k, (double)v / kGridUnit);
    }
}

// One CTA per q: partial[k][0] = sum over the present type pairs of
// f_ti(q) f_tj(q) sum_b (W_b g(r_b) + D_b h g'(r_b)), in FP64, with
// g(r) = sin(q r)/r, g'(r) = (q r cos(q r) - sin(q r)) / r^2 and, at r = 0,
// g = q, g' = 0.  sin/cos(q r_b) in FP32 with the rounding of q r_b folded in
// (r_b = b h is exact in double and carried as hi + lo).
__global__ void __launch_bounds__(256)
    forward_grid_eval_kernel(const DebyeArgs a, const double *hist, int nodes, float h,
                             unsigned type_mask)
{
    __shared__ double s_w[8];
    const int k = blockIdx.x;
    const float qk = a.q[k];
    const int T = a.n_types;
    double acc = 0.0;
    for (int idx = threadIdx.x; idx < T * T * nodes; idx += blockDim.x) {
        const int tp = idx / nodes, b = idx - tp * nodes;
        const int ti = tp / T, tj = tp - ti * T;
        if (tj < ti || !((type_mask >> ti) & 1u) || !((type_mask >> tj) & 1u))
            continue;
        const double *row = hist + (size_t)tp * 2 * nodes;
        const double W = row[b], D = row[nodes + b];
        if (W == 0.0 && D == 0.0)
            continue;
        double g, dg;
        if (b == 0) {
            g = qk;
            dg = 0.0;
        } else {
            const double rb = (double)b * (double)h;
            const float r_hi = (float)rb, r_lo = (float)(rb - (double)r_hi);
            const float x = qk * r_hi;
            const float x_lo = fmaf(qk, r_hi, -x) + qk * r_lo;
            float s, c;
            sincos_rr2(x, x_lo, s, c);
            // 1/r_b from the FP32 reciprocal with one Newton step in FP64
            const double y0 = (double)__frcp_rn(r_hi);
            const double rinv = y0 * (2.0 - rb * y0);
            g = (double)s * rinv;
            dg = ((double)qk * (double)c - g) * rinv;
        }
        const double f = (double)a.ff[(size_t)k * T + ti] * (double)a.ff[(size_t)k * T + tj];
        acc += f * (W * g + D * (double)h * dg);
    }
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1)
        acc += __shfl_xor_sync(0xffffffffu, acc, m);
    if ((threadIdx.x & 31) == 0)
        s_w[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w)
            s += s_w[w];
        a.partial[k] = s; // partial[k][0]: one part per q
    }
}

int forward_grid_max_nodes()
{
    // two 8-byte histograms per node in the deposit kernel's dynamic shared
    // memory, below the 227 KB a CTA may opt into (the static part is 2 KB)
    return (200 * 1024) / 16;
}

cudaError_t launch_forward_grid(const DebyeArgs &a, double *hist, int nodes, float h,
                                unsigned type_mask, cudaStream_t st)
{
    if (nodes < 2 || nodes > forward_grid_max_nodes() || a.n_types > 32)
        return cudaErrorInvalidValue;
    cudaError_t e =
        cudaMemsetAsync(hist, 0, sizeof(double) * 2 * (size_t)nodes * a.n_types * a.n_types, st);
    if (e != cudaSuccess)
        return e;
    if (a.n_items > 0) {
        const size_t smem = sizeof(unsigned long long) * 2 * (size_t)nodes;
        if (smem > 48 * 1024) {
            e = cudaFuncSetAttribute(forward_grid_deposit_kernel,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess)
                return e;
        }
        forward_grid_deposit_kernel<<<a.n_items, kBlockAtoms, smem, st>>>(a, hist, nodes, h,
                                                                          1.0f / h);
        count_launch();
        e = cudaGetLastError();
        if (e != cudaSuccess)
            return e;
    }
    forward_grid_eval_kernel<<<a.n_q, 256, 0, st>>>(a, hist, nodes, h, type_mask);
    count_launch();
    return cudaGetLastError();
}

} // namespace rsx
