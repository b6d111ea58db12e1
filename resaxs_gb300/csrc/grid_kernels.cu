// Forward on q grids without the uniform-step recurrence (non-uniform grids)
// through the gridded pair-distance distribution.  Written from scratch for
// this project.
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
//
// With the implicit water term a body's factor is f~ = f_t + w rsasa f_w, so
// f~_i f~_j = f_ti f_tj + w f_w (rsasa_i f_tj + rsasa_j f_ti) + w^2 f_w^2
// rsasa_i rsasa_j: the pairs deposit four histograms, weighted by 1, rsasa_i,
// rsasa_j and rsasa_i rsasa_j, and the per-q factors apply at evaluation.
#include "debye_device.cuh"

#include <algorithm>

namespace rsx {

constexpr double kGridUnit = 4294967296.0; // 2^32

__device__ __forceinline__ unsigned long long grid_fixed(float w)
{
    return (unsigned long long)__double2ll_rn((double)w * kGridUnit);
}

// Histograms per type pair: 1 without water, 4 with (weights 1, rsasa_i,
// rsasa_j, rsasa_i rsasa_j), each [2][nodes] (W then D).
template <bool WATER>
constexpr int kGridHists = WATER ? 4 : 1;

// One CTA per forward work item (one type pair): the item's pairs deposit into
// shared-memory histograms, which are then added to the type pair's FP64
// global histograms [n_types^2][hists][2][nodes].
template <bool WATER>
__global__ void __launch_bounds__(kBlockAtoms)
    forward_grid_deposit_kernel(const DebyeArgs a, double *hist, int nodes, float h, float inv_h)
{
    constexpr int NH = kGridHists<WATER>;
    extern __shared__ unsigned long long s_hist[]; // [NH][2][nodes]
    __shared__ float4 s_pos[kBlockAtoms];
    __shared__ float s_rs[WATER ? kBlockAtoms : 1];
    const int tid = threadIdx.x;
    for (int k = tid; k < NH * 2 * nodes; k += kBlockAtoms)
        s_hist[k] = 0ull;
    const PairItem it = a.items[blockIdx.x];
    const BlockDesc bi = a.blocks[it.bi];
    const int tj = a.blocks[it.bj_begin].type;
    const int i = bi.start + tid;
    const bool valid_i = tid < bi.len;
    const float4 pi = valid_i ? a.pos[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float rs_i = (WATER && valid_i) ? a.rsasa[i] : 0.f;

    for (int b = it.bj_begin; b < it.bj_end; ++b) {
        const BlockDesc bj = a.blocks[b];
        __syncthreads(); // also orders the histogram clearing before the first adds
        if (tid < bj.len) {
            s_pos[tid] = a.pos[bj.start + tid];
            if (WATER)
                s_rs[tid] = a.rsasa[bj.start + tid];
        }
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
            float m[NH];
            m[0] = 1.0f;
            if (WATER) {
                const float rs_j = s_rs[jj];
                m[1] = rs_i;
                m[2] = rs_j;
                m[3] = rs_i * rs_j;
            }
#pragma unroll
            for (int c = 0; c < NH; ++c) {
                unsigned long long *hc = s_hist + c * 2 * nodes;
                atomicAdd(&hc[n], grid_fixed(m[c] * h00));
                atomicAdd(&hc[n + 1], grid_fixed(m[c] * h01));
                atomicAdd(&hc[nodes + n], grid_fixed(m[c] * h10));
                atomicAdd(&hc[nodes + n + 1], grid_fixed(m[c] * h11));
            }
        }
    }
    __syncthreads();
    double *dst = hist + (size_t)(bi.type * a.n_types + tj) * NH * 2 * nodes;
    for (int k = tid; k < NH * 2 * nodes; k += kBlockAtoms) {
        const long long v = (long long)s_hist[k];
        if (v != 0)
            atomicAdd(dst + k, (double)v / kGridUnit);
    }
}

// g(q_k, r_b) = sin(q r_b)/r_b and h g'(q_k, r_b) = h (q r cos(q r) - sin(q r))
// / r^2 for every q and node, in FP64 ([2][n_q][nodes]); at r = 0, g = q and
// g' = 0.  sin/cos(q r_b) in FP32 with the rounding of q r_b folded in (r_b =
// b h is exact in double and carried as hi + lo); 1/r_b from the FP32
// reciprocal with one Newton step in FP64.
__global__ void __launch_bounds__(256)
    forward_grid_gtab_kernel(const DebyeArgs a, double *gtab, int nodes, float h)
{
    const size_t n = (size_t)a.n_q * nodes;
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n;
         idx += (size_t)gridDim.x * blockDim.x) {
        const int k = (int)(idx / nodes), b = (int)(idx - (size_t)k * nodes);
        const float qk = a.q[k];
        double g = qk, dg = 0.0;
        if (b > 0) {
            const double rb = (double)b * (double)h;
            const float r_hi = (float)rb, r_lo = (float)(rb - (double)r_hi);
            const float x = qk * r_hi;
            const float x_lo = fmaf(qk, r_hi, -x) + qk * r_lo;
            float s, c;
            sincos_rr2(x, x_lo, s, c);
            const double y0 = (double)__frcp_rn(r_hi);
            const double rinv = y0 * (2.0 - rb * y0);
            g = (double)s * rinv;
            dg = ((double)qk * (double)c - g) * rinv;
        }
        gtab[idx] = g;
        gtab[n + idx] = (double)h * dg;
    }
}

// One CTA per q: partial[k][0] = sum over the present type pairs (t_i <= t_j)
// of sum_c F_c(q) sum_b (W_cb g(q, r_b) + D_cb h g'(q, r_b)), in FP64, with
// F_0 = f_ti f_tj and, with water, F_1 = w f_w f_tj, F_2 = w f_w f_ti,
// F_3 = (w f_w)^2.  The node sums of a type pair are reduced over the CTA
// before its factors apply.
template <bool WATER>
__global__ void __launch_bounds__(256)
    forward_grid_eval_kernel(const DebyeArgs a, const double *hist, const double *gtab, int nodes,
                             unsigned type_mask)
{
    constexpr int NH = kGridHists<WATER>;
    __shared__ double s_w[8][NH];
    const int k = blockIdx.x;
    const int T = a.n_types;
    const size_t n = (size_t)a.n_q * nodes;
    const double *g = gtab + (size_t)k * nodes, *dg = gtab + n + (size_t)k * nodes;
    double acc = 0.0;
    for (int tp = 0; tp < T * T; ++tp) { // uniform over the CTA
        const int ti = tp / T, tj = tp - ti * T;
        if (tj < ti || !((type_mask >> ti) & 1u) || !((type_mask >> tj) & 1u))
            continue;
        const double *row = hist + (size_t)tp * NH * 2 * nodes;
        double part[NH];
#pragma unroll
        for (int c = 0; c < NH; ++c)
            part[c] = 0.0;
        for (int b = threadIdx.x; b < nodes; b += blockDim.x) {
            const double gb = g[b], dgb = dg[b];
#pragma unroll
            for (int c = 0; c < NH; ++c)
                part[c] = fma(row[c * 2 * nodes + b], gb, fma(row[c * 2 * nodes + nodes + b], dgb,
                                                            part[c]));
        }
#pragma unroll
        for (int c = 0; c < NH; ++c)
#pragma unroll
            for (int m = 16; m >= 1; m >>= 1)
                part[c] += __shfl_xor_sync(0xffffffffu, part[c], m);
        __syncthreads(); // the previous type pair's s_w is read
        if ((threadIdx.x & 31) == 0)
#pragma unroll
            for (int c = 0; c < NH; ++c)
                s_w[threadIdx.x >> 5][c] = part[c];
        __syncthreads();
        if (threadIdx.x == 0) {
            const double fi = a.ff[(size_t)k * T + ti], fj = a.ff[(size_t)k * T + tj];
            double F[NH];
            F[0] = fi * fj;
            if (WATER) {
                const double fw =
                    (double)a.water_weight * (double)a.ff[(size_t)k * T + a.water_index];
                F[1] = fw * fj;
                F[2] = fw * fi;
                F[3] = fw * fw;
            }
#pragma unroll
            for (int c = 0; c < NH; ++c) {
                double s = 0.0;
                for (int w = 0; w < (int)(blockDim.x >> 5); ++w)
                    s += s_w[w][c];
                acc += F[c] * s;
            }
        }
    }
    if (threadIdx.x == 0)
        a.partial[k] = acc; // partial[k][0]: one part per q
}

int forward_grid_hists(bool water) { return water ? kGridHists<true> : kGridHists<false>; }

int forward_grid_max_nodes(bool water)
{
    // 2 x hists 8-byte counters per node in the deposit kernel's dynamic
    // shared memory, below the 227 KB a CTA may opt into (static part < 3 KB)
    return (200 * 1024) / (16 * forward_grid_hists(water));
}

template <bool WATER>
static cudaError_t grid_launch(const DebyeArgs &a, double *hist, double *gtab, int nodes, float h,
                               unsigned type_mask, cudaStream_t st)
{
    cudaError_t e = cudaSuccess;
    if (a.n_items > 0) {
        const size_t smem = sizeof(unsigned long long) * kGridHists<WATER> * 2 * (size_t)nodes;
        if (smem > 48 * 1024) {
            e = cudaFuncSetAttribute(forward_grid_deposit_kernel<WATER>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess)
                return e;
        }
        forward_grid_deposit_kernel<WATER><<<a.n_items, kBlockAtoms, smem, st>>>(a, hist, nodes, h,
                                                                                 1.0f / h);
        count_launch();
        e = cudaGetLastError();
        if (e != cudaSuccess)
            return e;
    }
    const size_t n = (size_t)a.n_q * nodes;
    const int blocks = (int)std::min<size_t>((n + 255) / 256, 4096);
    forward_grid_gtab_kernel<<<blocks, 256, 0, st>>>(a, gtab, nodes, h);
    count_launch();
    e = cudaGetLastError();
    if (e != cudaSuccess)
        return e;
    forward_grid_eval_kernel<WATER><<<a.n_q, 256, 0, st>>>(a, hist, gtab, nodes, type_mask);
    count_launch();
    return cudaGetLastError();
}

size_t forward_grid_doubles(int n_types, int n_q, int nodes, bool water)
{
    return (size_t)forward_grid_hists(water) * 2 * nodes * n_types * n_types +
           2 * (size_t)n_q * nodes;
}

cudaError_t launch_forward_grid(const DebyeArgs &a, double *hist, int nodes, float h,
                                unsigned type_mask, bool water, cudaStream_t st)
{
    if (nodes < 2 || nodes > forward_grid_max_nodes(water) || a.n_types > 32 ||
        (water && !a.rsasa))
        return cudaErrorInvalidValue;
    const cudaError_t e =
        cudaMemsetAsync(hist, 0,
                        sizeof(double) * forward_grid_hists(water) * 2 * (size_t)nodes *
                            a.n_types * a.n_types,
                        st);
    if (e != cudaSuccess)
        return e;
    // the g tables follow the histograms in the same buffer
    double *gtab = hist + (size_t)forward_grid_hists(water) * 2 * nodes * a.n_types * a.n_types;
    return water ? grid_launch<true>(a, hist, gtab, nodes, h, type_mask, st)
                 : grid_launch<false>(a, hist, gtab, nodes, h, type_mask, st);
}

} // namespace rsx
