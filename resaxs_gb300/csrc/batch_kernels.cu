// Batched ensembles of conformations with uneven atom counts, for sm_103a.
//
// All members share the q grid and factor table; their bodies are
// concatenated (each member type-sorted within its own range) and their block
// tiles and work items are concatenated too, so a work item never mixes
// members.  One persistent kernel per pass walks the whole ensemble: every
// CTA repeatedly takes the next (item, q-slab) unit from an atomic counter
// (largest items first) and runs the same per-item code as the single-
// structure kernels (debye_device.cuh).  There is no waiting on other CTAs:
// the counter only hands out work, so a CTA finishes as soon as the units
// run out.
#include "debye_device.cuh"

#include <algorithm>
#include "rsx_batch_internal.h"

namespace rsx {

template <int QS, bool UNIFORM, bool WATER = false>
__global__ void __launch_bounds__(kBlockAtoms)
    batch_forward_kernel(const DebyeArgs a, const int *work_order, int n_units, int n_slabs,
                         int k_base, int *counter)
{
    __shared__ int s_w;
    for (;;) {
        if (threadIdx.x == 0)
            s_w = atomicAdd(counter, 1);
        __syncthreads();
        const int w = s_w;
        __syncthreads();
        if (w >= n_units)
            break;
        const int item = work_order[w / n_slabs];
        forward_item<QS, UNIFORM, WATER>(a, item, k_base + (w % n_slabs) * QS);
    }
}

// Chained forward (forward_chain_item) over work units (item, chain) handed
// out by the counter, largest items first; chain c starts at
// k_chain0 + c * chain_q.
template <int QT, bool SIGNED>
__global__ void __launch_bounds__(kBlockAtoms, 2)
    batch_chain_kernel(const DebyeArgs a, const int *work_order, int n_units, int n_chains,
                       int k_chain0, int chain_q, int n_main, int q_slots, int *counter)
{
    extern __shared__ __align__(16) unsigned char dsm[];
    __shared__ int s_w;
    for (;;) {
        if (threadIdx.x == 0)
            s_w = atomicAdd(counter, 1);
        __syncthreads();
        const int w = s_w;
        __syncthreads();
        if (w >= n_units)
            break;
        forward_chain_item<QT, SIGNED>(a, work_order[w / n_chains],
                                       k_chain0 + (w % n_chains) * chain_q, chain_q, n_main,
                                       q_slots, dsm);
    }
}

// Wide uniform slabs with the implicit water term, as forward_wide_water_kernel.
template <int QS, bool SIGNED>
__global__ void __launch_bounds__(kBlockAtoms, (QS <= 64 || !SIGNED) ? 3 : 2)
    batch_wide_water_kernel(const DebyeArgs a, const int *work_order, int n_units, int n_slabs,
                            int k_base, int *counter)
{
    __shared__ int s_w;
    for (;;) {
        if (threadIdx.x == 0)
            s_w = atomicAdd(counter, 1);
        __syncthreads();
        const int w = s_w;
        __syncthreads();
        if (w >= n_units)
            break;
        const int item = work_order[w / n_slabs];
        forward_wide_water_item<QS, SIGNED>(a, item, k_base + (w % n_slabs) * QS);
    }
}

// Wide uniform slabs (no water), as forward_wide_kernel (same register
// classes: 3 CTAs per SM for two plain pairs per step up to 128 q).
template <int QS, int IL, bool SIGNED = true>
__global__ void __launch_bounds__(kBlockAtoms,
                                  (IL == 2 && (QS <= 64 || (!SIGNED && QS <= 128))) ? 3 : 2)
    batch_wide_kernel(const DebyeArgs a, const int *work_order, int n_units, int n_slabs,
                      int k_base, int *counter)
{
    __shared__ int s_w;
    for (;;) {
        if (threadIdx.x == 0)
            s_w = atomicAdd(counter, 1);
        __syncthreads();
        const int w = s_w;
        __syncthreads();
        if (w >= n_units)
            break;
        const int item = work_order[w / n_slabs];
        forward_wide_item<QS, IL, SIGNED>(a, item, k_base + (w % n_slabs) * QS);
    }
}

template <int QS, bool UNIFORM, bool SMALL = false>
__global__ void __launch_bounds__(kBlockAtoms, UNIFORM ? 4 : 1)
    batch_adjoint_kernel(const DebyeArgs a, const int *work_order, int n_units, int n_slabs,
                         int *counter)
{
    __shared__ int s_w;
    for (;;) {
        if (threadIdx.x == 0)
            s_w = atomicAdd(counter, 1);
        __syncthreads();
        const int w = s_w;
        __syncthreads();
        if (w >= n_units)
            break;
        adjoint_item<QS, UNIFORM, false, SMALL>(a, work_order[w], n_slabs);
    }
}

__global__ void __launch_bounds__(256) batch_assemble_kernel(const BatchAssembleArgs a)
{
    __shared__ double s_w[8];
    const int k = blockIdx.x, m = blockIdx.y;
    const int2 rg = a.item_range[m];
    const double *row = a.partial + (size_t)k * a.n_items;
    double s = 0.0;
    // at q = 0 the cross sums are not used (the row may not be written)
    const int end = a.q[k] != 0.f ? rg.y : rg.x;
    for (int x = rg.x + threadIdx.x; x < end; x += blockDim.x)
        s += row[x];
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1)
        s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0)
        s_w[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x != 0)
        return;
    double cross = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w)
        cross += s_w[w];
    const double q = a.q[k];
    double self = 0.0, sumf = 0.0;
    const float *ff = a.ff + (size_t)k * a.n_types;
    const int *cnt = a.type_count + (size_t)m * a.n_types;
    // f~_i = f_t + w rsasa_i f_w: sum f~^2 = sum f_t^2 + 2 w f_w sum_t f_t S_t +
    // (w f_w)^2 sum rsasa^2, sum f~ = sum f_t + w f_w sum rsasa (assemble_kernel)
    const double fw = a.has_water ? (double)(a.water_weight * ff[a.water_index]) : 0.0;
    for (int t = 0; t < a.n_types; ++t) {
        self += cnt[t] * (double)ff[t] * ff[t];
        sumf += cnt[t] * (double)ff[t];
        if (a.has_water)
            self += 2.0 * fw * ff[t] * a.rsasa_sum[(size_t)m * a.n_types + t];
    }
    if (a.has_water) {
        self += fw * fw * a.rsasa_sq[m];
        sumf += fw * a.rsasa_tot[m];
    }
    const double iq = (q != 0.0) ? self + 2.0 * cross / q : sumf * sumf;
    a.iq64[(size_t)m * a.n_q + k] = iq;
    a.iq32[(size_t)m * a.n_q + k] = (float)iq;
}

__global__ void __launch_bounds__(256) batch_loss_kernel(const BatchLossArgs a)
{
    __shared__ double s_w[8];
    const int m = blockIdx.x;
    double c2 = 0.0;
    for (int k = threadIdx.x; k < a.n_q; k += blockDim.x) {
        const size_t o = (size_t)m * a.n_q + k;
        const double sg = a.sigma[o];
        const double d = (a.iq64[o] - a.target[o]) / sg;
        c2 += d * d;
        a.lambda[o] = (float)(2.0 * d / sg);
    }
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1)
        c2 += __shfl_xor_sync(0xffffffffu, c2, o);
    if ((threadIdx.x & 31) == 0)
        s_w[threadIdx.x >> 5] = c2;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w)
            t += s_w[w];
        a.chi2[m] = t;
    }
}

template <int QS, bool U, bool W = false>
static cudaError_t fwd_launch(const DebyeArgs &a, const int *order, int n_items, int n_slabs,
                              int k_base, int *counter, int grid, cudaStream_t st)
{
    batch_forward_kernel<QS, U, W><<<grid, kBlockAtoms, 0, st>>>(a, order, n_items * n_slabs,
                                                                 n_slabs, k_base, counter);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_batch_forward(const DebyeArgs &a, const int *work_order, int n_work_items,
                                 int q_slab, int n_slabs, int k_base, bool uniform,
                                 int *counter, int grid, cudaStream_t st, bool water)
{
    if (n_work_items == 0 || n_slabs == 0)
        return cudaSuccess;
    if (water) { // two accumulator sets per thread: 8 or 16 q per slab
        if (q_slab == 8)
            return uniform ? fwd_launch<8, true, true>(a, work_order, n_work_items, n_slabs,
                                                       k_base, counter, grid, st)
                           : fwd_launch<8, false, true>(a, work_order, n_work_items, n_slabs,
                                                        k_base, counter, grid, st);
        if (q_slab == 16)
            return uniform ? fwd_launch<16, true, true>(a, work_order, n_work_items, n_slabs,
                                                        k_base, counter, grid, st)
                           : fwd_launch<16, false, true>(a, work_order, n_work_items, n_slabs,
                                                         k_base, counter, grid, st);
        return cudaErrorInvalidValue;
    }
#define RSX_BF(QS)                                                                         \
    return uniform ? fwd_launch<QS, true>(a, work_order, n_work_items, n_slabs, k_base,    \
                                          counter, grid, st)                               \
                   : fwd_launch<QS, false>(a, work_order, n_work_items, n_slabs, k_base,   \
                                           counter, grid, st)
    switch (q_slab) {
    case 8:
        RSX_BF(8);
    case 16:
        RSX_BF(16);
    case 32:
        RSX_BF(32);
    default: // 64 and wider: launch_batch_forward_wide
        return cudaErrorInvalidValue;
    }
#undef RSX_BF
}

template <class K>
static int occupancy_grid(K kfn, size_t smem, int sms);


template <int QS>
static cudaError_t wide_batch_water_launch(const DebyeArgs &a, const int *order, int n_items,
                                           int n_slabs, int k_base, int *counter, int sms,
                                           cudaStream_t st)
{
    if constexpr (QS > 128) {
        return cudaErrorInvalidValue; // the water slabs stop at 128 q
    } else {
        auto kfn = a.small_theta >= 2 ? batch_wide_water_kernel<QS, false>
                                      : batch_wide_water_kernel<QS, true>;
        const int grid = std::min(occupancy_grid(kfn, 0, sms), n_items * n_slabs);
        kfn<<<grid, kBlockAtoms, 0, st>>>(a, order, n_items * n_slabs, n_slabs, k_base, counter);
        count_launch();
        return cudaGetLastError();
    }
}

template <int QS>
static cudaError_t wide_batch_launch(const DebyeArgs &a, const int *order, int n_items,
                                     int n_slabs, int k_base, int *counter, int sms,
                                     cudaStream_t st, bool main = false, bool water = false)
{
    if (water)
        return wide_batch_water_launch<QS>(a, order, n_items, n_slabs, k_base, counter, sms, st);
    // instantiations as in the single-structure launcher (four pairs per step
    // in the main slabs of 128 q and more when the tuned tile shape says so)
    auto kfn = a.small_theta >= 2 ? batch_wide_kernel<QS, 2, false> : batch_wide_kernel<QS, 2, true>;
    if constexpr (QS >= 128) {
        if (main && a.pairs4)
            kfn = a.small_theta >= 2 ? batch_wide_kernel<QS, 4, false>
                                     : batch_wide_kernel<QS, 4, true>;
    }
    const int grid = std::min(occupancy_grid(kfn, 0, sms), n_items * n_slabs);
    kfn<<<grid, kBlockAtoms, 0, st>>>(a, order, n_items * n_slabs, n_slabs, k_base, counter);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_batch_forward_wide(const DebyeArgs &a, const int *work_order,
                                      int n_work_items, int q_slab, int *counters, int sms,
                                      cudaStream_t st, bool water)
{
    if (n_work_items == 0)
        return cudaSuccess;
    const WidePlan p = wide_plan(a.n_q, water ? std::min(q_slab, 128) : q_slab);
    if (p.full > 0) {
        cudaError_t e;
        e = p.main == 64    ? wide_batch_launch<64>(a, work_order, n_work_items, p.full, 0,
                                                    counters, sms, st, false, water)
            : p.main == 112 ? wide_batch_launch<112>(a, work_order, n_work_items, p.full, 0,
                                                     counters, sms, st, false, water)
            : p.main == 192 ? wide_batch_launch<192>(a, work_order, n_work_items, p.full, 0,
                                                     counters, sms, st, true, water)
                            : wide_batch_launch<128>(a, work_order, n_work_items, p.full, 0,
                                                     counters, sms, st, true, water);
        if (e != cudaSuccess)
            return e;
    }
    if (p.tail_len == 0)
        return cudaSuccess;
#define RSX_BW(QS)                                                                         \
    return wide_batch_launch<QS>(a, work_order, n_work_items, 1, p.tail_k0, counters + 1, sms, \
                                 st, false, water)
    switch (p.tail_w / 16) {
    case 1:
        RSX_BW(16);
    case 2:
        RSX_BW(32);
    case 3:
        RSX_BW(48);
    case 4:
        RSX_BW(64);
    case 5:
        RSX_BW(80);
    case 6:
        RSX_BW(96);
    case 7:
        RSX_BW(112);
    default:
        RSX_BW(128);
    }
#undef RSX_BW
}

template <int QT>
static cudaError_t batch_chain_launch(const DebyeArgs &a, const int *order, int n_items,
                                      int n_chains, int k_chain0, int n_main, int *counter,
                                      int sms, cudaStream_t st)
{
    const int chain_q = n_main * kChainMain + QT;
    const int q_slots = n_main * kChainMain + (QT + 31) / 32 * 32;
    const size_t smem = chain_smem_bytes(q_slots);
    auto kfn = a.small_theta >= 2 ? batch_chain_kernel<QT, false> : batch_chain_kernel<QT, true>;
    if (smem > 32 * 1024) { // with the static arrays past the 48 KB default
        const cudaError_t e =
            cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess)
            return e;
    }
    const int grid = std::min(occupancy_grid(kfn, smem, sms), n_items * n_chains);
    kfn<<<grid, kBlockAtoms, smem, st>>>(a, order, n_items * n_chains, n_chains, k_chain0, chain_q,
                                        n_main, q_slots, counter);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_batch_forward_chain(const DebyeArgs &a, const int *work_order,
                                       int n_work_items, int *counters, int sms, cudaStream_t st)
{
    if (n_work_items == 0)
        return cudaSuccess;
    const ChainPlan p = chain_plan(a.n_q);
    if (p.full > 0) {
        const cudaError_t e = batch_chain_launch<0>(a, work_order, n_work_items, p.full, 0,
                                                    kChainMaxMain, counters, sms, st);
        if (e != cudaSuccess)
            return e;
    }
    if (!p.rest)
        return cudaSuccess;
    // a rest of one tail slab only: the slab kernels (a chain pays its
    // sub-tile reductions for nothing when no slab follows)
    if (p.rest_main == 0 && p.rest_tail <= 128) {
#define RSX_BT(QS)                                                                         \
    return wide_batch_launch<QS>(a, work_order, n_work_items, 1, p.rest_k0, counters + 1, sms, st)
        switch ((p.rest_tail + 15) / 16) { // a tail of 8 runs as 16
        case 1: RSX_BT(16);
        case 2: RSX_BT(32);
        case 3: RSX_BT(48);
        case 4: RSX_BT(64);
        case 5: RSX_BT(80);
        case 6: RSX_BT(96);
        case 7: RSX_BT(112);
        default: RSX_BT(128);
        }
#undef RSX_BT
    }
#define RSX_BC(QT)                                                                         \
    return batch_chain_launch<QT>(a, work_order, n_work_items, 1, p.rest_k0, p.rest_main,   \
                                  counters + 1, sms, st)
    if (p.rest_tail == 8)
        RSX_BC(8);
    switch (p.rest_tail / 16) {
    case 0: RSX_BC(0);
    case 1: RSX_BC(16);
    case 2: RSX_BC(32);
    case 3: RSX_BC(48);
    case 4: RSX_BC(64);
    case 5: RSX_BC(80);
    case 6: RSX_BC(96);
    case 7: RSX_BC(112);
    case 8: RSX_BC(128);
    case 9: RSX_BC(144);
    case 10: RSX_BC(160);
    case 11: RSX_BC(176);
    default:
        return cudaErrorInvalidValue;
    }
#undef RSX_BC
}

template <int QS, bool U>
static cudaError_t adj_launch(const DebyeArgs &a, const int *order, int n_items, int *counter,
                              int grid, cudaStream_t st)
{
    const int n_slabs = (a.n_q + QS - 1) / QS;
    const size_t smem = adjoint_smem_bytes(a.n_q, QS, U, false);
    auto kfn = (U && a.small_theta >= 1) ? batch_adjoint_kernel<QS, U, true> : batch_adjoint_kernel<QS, U, false>;
    if (smem > 48 * 1024) {
        cudaError_t e =
            cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess)
            return e;
    }
    kfn<<<grid, kBlockAtoms, smem, st>>>(a, order, n_items, n_slabs, counter);
    count_launch();
    return cudaGetLastError();
}

// Persistent pair pass of the adjoint through tabulated pair functions: each
// unit is one adjoint item; its member's tables are selected by PairItem::pad.
__global__ void __launch_bounds__(kBlockAtoms)
    batch_adjoint_table_kernel(const DebyeArgs a, const int *work_order, int n_units, int *counter)
{
    __shared__ int s_w;
    for (;;) {
        if (threadIdx.x == 0)
            s_w = atomicAdd(counter, 1);
        __syncthreads();
        const int w = s_w;
        __syncthreads();
        if (w >= n_units)
            break;
        adjoint_table_item<4>(a, work_order[w]);
    }
}

cudaError_t launch_batch_adjoint_table(const DebyeArgs &a, const int *work_order,
                                       int n_work_items, int *counter, int grid, cudaStream_t st)
{
    if (n_work_items == 0)
        return cudaSuccess;
    batch_adjoint_table_kernel<<<grid, kBlockAtoms, 0, st>>>(a, work_order, n_work_items, counter);
    count_launch();
    return cudaGetLastError();
}

int batch_adjoint_table_grid(int sms)
{
    return occupancy_grid(batch_adjoint_table_kernel, 0, sms);
}

cudaError_t launch_batch_adjoint(const DebyeArgs &a, const int *work_order, int n_work_items,
                                 int q_slab, bool uniform, int *counter, int grid,
                                 cudaStream_t st)
{
    if (n_work_items == 0)
        return cudaSuccess;
    const int qs = q_slab > 32 ? 32 : q_slab; // the adjoint keeps two sums, not QS
    switch (qs) {
    case 8:
        return uniform ? adj_launch<8, true>(a, work_order, n_work_items, counter, grid, st)
                       : adj_launch<8, false>(a, work_order, n_work_items, counter, grid, st);
    case 16:
        return uniform ? adj_launch<16, true>(a, work_order, n_work_items, counter, grid, st)
                       : adj_launch<16, false>(a, work_order, n_work_items, counter, grid, st);
    default:
        return uniform ? adj_launch<32, true>(a, work_order, n_work_items, counter, grid, st)
                       : adj_launch<32, false>(a, work_order, n_work_items, counter, grid, st);
    }
}

cudaError_t launch_batch_assemble(const BatchAssembleArgs &a, cudaStream_t st)
{
    if (a.n_members == 0)
        return cudaSuccess;
    batch_assemble_kernel<<<dim3(a.n_q, a.n_members), 256, 0, st>>>(a);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_batch_loss(const BatchLossArgs &a, cudaStream_t st)
{
    if (a.n_members == 0)
        return cudaSuccess;
    batch_loss_kernel<<<a.n_members, 256, 0, st>>>(a);
    count_launch();
    return cudaGetLastError();
}

template <class K>
static int occupancy_grid(K kfn, size_t smem, int sms)
{
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kfn, kBlockAtoms, smem) !=
            cudaSuccess ||
        per_sm < 1)
        per_sm = 1;
    return per_sm * sms;
}

int batch_forward_grid(int q_slab, bool uniform, int sms, bool water)
{
    if (water && q_slab <= 8)
        return uniform ? occupancy_grid(batch_forward_kernel<8, true, true>, 0, sms)
                       : occupancy_grid(batch_forward_kernel<8, false, true>, 0, sms);
    if (water)
        return uniform ? occupancy_grid(batch_forward_kernel<16, true, true>, 0, sms)
                       : occupancy_grid(batch_forward_kernel<16, false, true>, 0, sms);
    switch (q_slab) {
    case 8:
        return uniform ? occupancy_grid(batch_forward_kernel<8, true>, 0, sms)
                       : occupancy_grid(batch_forward_kernel<8, false>, 0, sms);
    case 16:
        return uniform ? occupancy_grid(batch_forward_kernel<16, true>, 0, sms)
                       : occupancy_grid(batch_forward_kernel<16, false>, 0, sms);
    case 32:
        return uniform ? occupancy_grid(batch_forward_kernel<32, true>, 0, sms)
                       : occupancy_grid(batch_forward_kernel<32, false>, 0, sms);
    case 64:
        return uniform ? occupancy_grid(batch_wide_kernel<64, 2, true>, 0, sms)
                       : occupancy_grid(batch_forward_kernel<32, false>, 0, sms);
    default:
        return uniform ? occupancy_grid(batch_wide_kernel<112, 2, true>, 0, sms)
                       : occupancy_grid(batch_forward_kernel<32, false>, 0, sms);
    }
}

int batch_adjoint_grid(int q_slab, bool uniform, int n_q, int sms)
{
    const int qs = q_slab > 32 ? 32 : (q_slab < 8 ? 8 : q_slab);
    const size_t smem = adjoint_smem_bytes(n_q, qs, uniform, false);
    if (qs == 8)
        return uniform ? occupancy_grid(batch_adjoint_kernel<8, true>, smem, sms)
                       : occupancy_grid(batch_adjoint_kernel<8, false>, smem, sms);
    if (qs == 16)
        return uniform ? occupancy_grid(batch_adjoint_kernel<16, true>, smem, sms)
                       : occupancy_grid(batch_adjoint_kernel<16, false>, smem, sms);
    return uniform ? occupancy_grid(batch_adjoint_kernel<32, true>, smem, sms)
                   : occupancy_grid(batch_adjoint_kernel<32, false>, smem, sms);
}

} // namespace rsx
