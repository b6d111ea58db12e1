// Adjoint kernel launches (dL/dx from dL/dI(q) in one pair pass), split from
// debye_kernels.cu so that the two translation units compile in parallel.
// The per-item device code is in debye_device.cuh.
#include "debye_device.cuh"

namespace rsx {

// ----------------------------------------------------------------------------
// adjoint: grad_i = sum_j G_ij (x_i - x_j),
//   G_ij = 2/r^2 sum_q lambda_q f_i f_j (cos(q r) - sinc(q r))
// Each pair is visited once (upper triangle); the J side of every pair is
// summed over the warp with shuffles, accumulated in shared memory and
// flushed to the FP64 gradient once per J-block.  The thread runs the whole
// q range for each pair (slab by slab, all in registers), so the gradient of
// a pair is complete before it is scattered.
// ----------------------------------------------------------------------------

// The uniform form: 4 CTAs per SM (8 pairs per thread step need 128 registers).
template <int QS, bool UNIFORM, bool WATER, bool SMALL = false>
__global__ void __launch_bounds__(kBlockAtoms, (UNIFORM && !WATER) ? 4 : 1)
    adjoint_kernel(const DebyeArgs a, int n_slabs)
{
    adjoint_item<QS, UNIFORM, WATER, SMALL>(a, blockIdx.x, n_slabs);
}

template <int QS>
static cudaError_t adjoint_qs(const DebyeArgs &a, bool uniform, bool water, cudaStream_t st)
{
    const int n_slabs = (a.n_q + QS - 1) / QS;
    const size_t smem = adjoint_smem_bytes(a.n_q, QS, uniform, water);
    const dim3 grid(a.n_items);
    cudaError_t e = cudaSuccess;
#define RSX_ADJ_SMALL()                                                                    \
    do {                                                                                   \
        auto kfn = adjoint_kernel<QS, true, false, true>;                                  \
        if (smem > 48 * 1024)                                                              \
            e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize,     \
                                     (int)smem);                                           \
        if (e == cudaSuccess)                                                              \
            kfn<<<grid, kBlockAtoms, smem, st>>>(a, n_slabs);                              \
    } while (0)
#define RSX_ADJ(U, W)                                                                      \
    do {                                                                                   \
        auto kfn = adjoint_kernel<QS, U, W>;                                               \
        if (smem > 48 * 1024)                                                              \
            e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize,     \
                                     (int)smem);                                           \
        if (e == cudaSuccess)                                                              \
            kfn<<<grid, kBlockAtoms, smem, st>>>(a, n_slabs);                              \
    } while (0)
    if (uniform && !water && a.small_theta >= 1)
        RSX_ADJ_SMALL();
    else if (uniform && !water)
        RSX_ADJ(true, false);
    else if (uniform && water)
        RSX_ADJ(true, true);
    else if (!uniform && !water)
        RSX_ADJ(false, false);
    else
        RSX_ADJ(false, true);
#undef RSX_ADJ
#undef RSX_ADJ_SMALL
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
    switch (q_slab > 32 ? 32 : q_slab) { // the adjoint walks all q per pair in 32-q slabs
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

// ----------------------------------------------------------------------------
// adjoint through tabulated pair functions (debye_device.cuh): the table of
// every present type pair (t_i <= t_j), then one pair pass
// ----------------------------------------------------------------------------

// One warp per node; grid (nodes / 4, n_types * n_types, members): member
// m's tables from its dL/dI row lambda + m * n_q.  Whole warps return
// together (the node sum shuffles over the warp).
template <bool WATER>
__global__ void __launch_bounds__(128)
    adjoint_table_kernel(const DebyeArgs a, float4 *tab, unsigned type_mask)
{
    constexpr int NT = kTableEntries<WATER>;
    const int lane = threadIdx.x & 31;
    const int b = blockIdx.x * 4 + (threadIdx.x >> 5);
    const int ti = blockIdx.y / a.n_types, tj = blockIdx.y % a.n_types, m = blockIdx.z;
    if (b >= a.adj_nodes || tj < ti || !((type_mask >> ti) & 1u) || !((type_mask >> tj) & 1u))
        return;
    const float h = a.adj_geom ? a.adj_geom[0] : a.adj_h;
    const size_t tp = (size_t)m * a.n_types * a.n_types + (size_t)(ti * a.n_types + tj);
#pragma unroll
    for (int c = 0; c < NT; ++c) {
        const float4 v = adjoint_table_node(a, a.lambda + (size_t)m * a.n_q, ti, tj, b, h, lane, c);
        if (lane == 0)
            tab[(tp * a.adj_nodes + b) * NT + c] = v;
    }
}

template <int IL, bool WATER>
__global__ void __launch_bounds__(kBlockAtoms) adjoint_pairs_table_kernel(const DebyeArgs a)
{
    adjoint_table_item<IL, WATER>(a, blockIdx.x);
}

cudaError_t launch_adjoint_tables(const DebyeArgs &a, float4 *tab, unsigned type_mask,
                                  int n_members, cudaStream_t st)
{
    if (a.n_types > 32 || a.adj_nodes < 2 || n_members < 1 || n_members > 65535)
        return cudaErrorInvalidValue;
    const dim3 g((a.adj_nodes + 3) / 4, a.n_types * a.n_types, n_members);
    adjoint_table_kernel<false><<<g, 128, 0, st>>>(a, tab, type_mask);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_adjoint_table(const DebyeArgs &a, float4 *tab, unsigned type_mask, bool water,
                                 cudaStream_t st)
{
    if (a.n_items == 0)
        return cudaSuccess;
    if (a.n_types > 32 || a.adj_nodes < 2 || (water && !a.rsasa))
        return cudaErrorInvalidValue;
    const dim3 g((a.adj_nodes + 3) / 4, a.n_types * a.n_types, 1);
    if (water)
        adjoint_table_kernel<true><<<g, 128, 0, st>>>(a, tab, type_mask);
    else
        adjoint_table_kernel<false><<<g, 128, 0, st>>>(a, tab, type_mask);
    count_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return e;
    if (water)
        adjoint_pairs_table_kernel<4, true><<<a.n_items, kBlockAtoms, 0, st>>>(a);
    else
        adjoint_pairs_table_kernel<4, false><<<a.n_items, kBlockAtoms, 0, st>>>(a);
    count_launch();
    return cudaGetLastError();
}

} // namespace rsx
