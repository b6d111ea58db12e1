// Debye pair kernels for sm_103a: forward I(q), incremental delta I(q) and
// the adjoint dL/dx, with their launchers.  Written from scratch for this
// project; the per-item device code is in debye_device.cuh.
//
// Common structure
//  * Bodies are stored in type-sorted order and cut into block tiles of at
//    most 128 bodies of one type (BlockDesc), so every (I-block, J-block) pair
//    of tiles has a single pair of form factors F[q][t_i] * F[q][t_j].
//  * One CTA of 128 threads owns an I-block (one body per thread) and streams
//    its J-blocks through shared memory with one float4 load per thread.
//  * A CTA covers a slab of consecutive q values.  On a uniform q grid the
//    per-pair values sin(q_k r)/r come from Reinsch's two-term recurrence
//    (3 FP32 ops per pair*q with the accumulation), seeded per pair and slab
//    from the range-reduced FP32 sin/cos of rsx_math.cuh; the wide forward
//    kernels run 64..192 q per seed following the slab plan of wide_plan(),
//    and the delta kernel (delta_chain_kernel) runs a chain of two slabs of up
//    to 112 q on one seed, with the even and odd q of a slab as two
//    sequences of step 2 theta packed in float2 lanes, so that each FP32x2
//    instruction advances both.  Non-uniform grids and water use
//    forward_kernel / delta_kernel (8..32 q per slab, sin/cos per pair*q).
//    sinc(q r) = (sin(q r)/r) / q: the 1/q factor is applied once per q in FP64
//    when the curve is assembled.
//  * Per-thread sums: FP32 over one J-block, then reduce-scattered over the
//    warp into FP64 (wide kernels) or folded into a Kahan accumulator per q
//    (general kernels).  Across warps and CTAs: FP64.
//  * The adjoint steps sin and cos(q r - theta/2) together (the magic-circle
//    form, two pairs per FP32x2 instruction) and sums both sides of every
//    pair's gradient; see debye_device.cuh.
#include "debye_device.cuh"

#include <algorithm>
#include <atomic>

namespace rsx {

static std::atomic<unsigned long long> g_launches{0};
void count_launch(int n) { g_launches += (unsigned long long)n; }
unsigned long long launch_count() { return g_launches.load(); }

template <int QS, bool UNIFORM, bool WATER>
__global__ void __launch_bounds__(kBlockAtoms) forward_kernel(const DebyeArgs a)
{
    forward_item<QS, UNIFORM, WATER>(a, blockIdx.x, a.k_base + blockIdx.y * QS);
}

// two pairs per step up to 64 q, and plain up to 128 q: <= 168 registers,
// 3 CTAs per SM; the rest (signed above 64 q, every instantiation above 128 q,
// four pairs per step): <= 255, 2 CTAs per SM
template <int QS, int IL, bool SIGNED>
__global__ void __launch_bounds__(kBlockAtoms,
                                  (IL == 2 && (QS <= 64 || (!SIGNED && QS <= 128))) ? 3 : 2)
    forward_wide_kernel(const DebyeArgs a)
{
    forward_wide_item<QS, IL, SIGNED>(a, blockIdx.x, a.k_base + blockIdx.y * QS);
}

// the same with the implicit water term (one more FP32x2 FMA per step)
template <int QS, bool SIGNED>
__global__ void __launch_bounds__(kBlockAtoms, (QS <= 64 || !SIGNED) ? 3 : 2)
    forward_wide_water_kernel(const DebyeArgs a)
{
    forward_wide_water_item<QS, SIGNED>(a, blockIdx.x, a.k_base + blockIdx.y * QS);
}

// ----------------------------------------------------------------------------
// assemble I(q) = self(q) + 2 * cross(q) / q  (q = 0: (sum f)^2)
// ----------------------------------------------------------------------------

__global__ void __launch_bounds__(256) assemble_kernel(const AssembleArgs a)
{
    __shared__ double s_w[8];
    const int k = blockIdx.x;
    if (k >= a.n_q) { // the moved bodies' new positions (incremental mode)
        const int m = (k - a.n_q) * blockDim.x + threadIdx.x;
        if (m < a.apply_k)
            a.apply_pos[a.apply_idx[m]] = a.apply_new[m];
        return;
    }
    double s = 0.0;
    const double *row = a.partial + (size_t)k * a.n_parts;
    // at q = 0 the cross sums are not used (the row may not be written)
    const int n_read = a.q[k] != 0.f ? a.n_parts : 0;
    for (int x = threadIdx.x; x < n_read; x += blockDim.x)
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

// Slot in the moved list of this thread's body of static block `by` (-1:
// static or past the block), found by scanning the moved list into shared
// memory (k <= n / 3 on this path; the indices are distinct).  No device
// state outlives the step.
__device__ __forceinline__ int moved_slot_of(const DeltaArgs &a, const BlockDesc &by, int *s_slot)
{
    const int tid = threadIdx.x;
    s_slot[tid] = -1;
    __syncthreads();
    for (int m = tid; m < a.k; m += kBlockAtoms) {
        const int i = a.moved_idx[m] - by.start;
        if (i >= 0 && i < by.len)
            s_slot[i] = m;
    }
    __syncthreads();
    return tid < by.len ? s_slot[tid] : -1;
}

template <int QS, bool UNIFORM>
__global__ void __launch_bounds__(kBlockAtoms) delta_kernel(const DeltaArgs a)
{
    __shared__ float4 s_new[kBlockAtoms], s_old[kBlockAtoms];
    __shared__ int s_idx[kBlockAtoms], s_slot[kBlockAtoms];
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
    const int slot = moved_slot_of(a, by, s_slot);
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
                // the old pair is seeded with -1/r so that the two chains
                // accumulate new - old directly
                const PairSeed pn = pair_seed(q0, dq, rn, scn);
                const PairSeed po = pair_seed(q0, dq, ro, -sco);
                float dummy[1];
                if (!pn.big && !po.big) {
                    pair2_slab<QS>(pn, po, S);
                } else {
                    pair_slab<QS, false>(pn, 0.f, S, dummy);
                    pair_slab<QS, false>(po, 0.f, S, dummy);
                }
            } else {
#pragma unroll
                for (int k = 0; k < QS; ++k) {
                    float s1, c1, s2, c2;
                    sincos_prod(s_q[k], rn, s1, c1);
                    sincos_prod(s_q[k], ro, s2, c2);
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

// Incremental delta on a uniform grid.  A CTA takes one static block and one
// group of moved tiles over a chain of two slabs, [k0, k0 + Q1) and
// [k0 + Q1, k0 + Q1 + Q2) (Q2 = 0: one slab), so each pair chain (new and
// old position of the moved body) is seeded once per Q1 + Q2 q: its
// recurrence state after the first slab (s, d of both chains, lam with the
// sign) waits in shared memory while the first slab's sums are reduced, then
// runs on through the second.  Per tile the warp sums the FP32 pair sums of
// its threads through shared memory (warp_sum_rows), lane L receiving q index
// 32c + L, applies the tile's factor f_x(q) to the sum and adds it to FP64
// lane accumulators; the two chains of a pair (new position, old position
// seeded with -1/r) run interleaved.  Tiles hold at most kDeltaTile moved
// bodies of one type.  Dynamic shared memory: delta_chain_smem(Q2) bytes.
__host__ __device__ constexpr size_t delta_chain_smem(int q2)
{
    return (q2 > 0 ? sizeof(float2) * kDeltaTile * 5 * kBlockAtoms : 0) +
           sizeof(float) * (kBlockAtoms / 32) * 32 * kSumStride;
}

template <int Q1, int Q2, bool SMALL>
__global__ void __launch_bounds__(kBlockAtoms, 3) delta_chain_kernel(const DeltaArgs a,
                                                                    int k_base)
{
    static_assert(Q1 % 16 == 0 && Q2 % 8 == 0 && Q1 <= 112 && Q2 <= 112, "chain slabs");
    constexpr int QP1 = WideSlab<Q1>::QP, NR1 = WideSlab<Q1>::NR;
    constexpr int QP2 = Q2 > 0 ? WideSlab<Q2>::QP : 0, NR2 = QP2 / 32;
    constexpr int T = kDeltaTile;
    constexpr size_t kStateBytes = Q2 > 0 ? sizeof(float2) * T * 5 * kBlockAtoms : 0;
    static_assert(sizeof(double) * (kBlockAtoms / 32) * (QP1 + QP2) <= delta_chain_smem(Q2),
                  "final sums fit the dynamic buffer");
    __shared__ float4 s_new[T], s_old[T];
    __shared__ int s_idx[T], s_slot[kBlockAtoms];
    __shared__ float s_fx[QP1 + QP2];
    // dynamic: chain states between the slabs ([body][5][thread]) and the
    // warps' summation buffers; after the tiles, the final cross-warp sums
    extern __shared__ __align__(16) unsigned char dsm[];
    float2 *u_st = reinterpret_cast<float2 *>(dsm);
    double(*u_red)[QP1 + QP2] = reinterpret_cast<double(*)[QP1 + QP2]>(dsm);

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    float *sum_buf = reinterpret_cast<float *>(dsm + kStateBytes) + warp * 32 * kSumStride;
    const BlockDesc by = a.blocks[blockIdx.x];
    const int k0 = k_base + blockIdx.y * (Q1 + Q2);
    const int group = blockIdx.z, n_groups = gridDim.z;
    const int y = by.start + tid;
    const bool valid = tid < by.len;
    const float4 py_old = valid ? a.pos_old[y] : make_float4(0.f, 0.f, 0.f, 0.f);
    const int slot = moved_slot_of(a, by, s_slot);
    const float4 py_new = slot >= 0 ? a.moved_new[slot] : py_old;
    // pairs with a static body are met once (weight 1); pairs inside the moved
    // list are met from both ends (weight 1/2 each)
    const float mult = !valid ? 0.f : (slot >= 0 ? 0.5f : 1.0f);
    const float q0 = a.q[k0];
    const float dq = a.dq;

    double acc1[NR1], acc2[NR2 > 0 ? NR2 : 1];
#pragma unroll
    for (int c = 0; c < NR1; ++c)
        acc1[c] = 0.0;
#pragma unroll
    for (int c = 0; c < NR2; ++c)
        acc2[c] = 0.0;
    for (int r = 0;; ++r) {
        // snake order over the rounds keeps the groups' totals close (tiles
        // come longest first)
        const int mt = r * n_groups + ((r & 1) ? n_groups - 1 - group : group);
        if (mt >= a.n_mtiles)
            break;
        const BlockDesc tile = a.mtiles[mt];
        const int len = min(tile.len, T);
        __syncthreads();
        if (tid < len) {
            const int m = tile.start + tid;
            const int idx = a.moved_idx[m];
            s_new[tid] = a.moved_new[m];
            s_old[tid] = a.pos_old[idx];
            s_idx[tid] = idx;
        }
        for (int k = tid; k < QP1 + QP2; k += kBlockAtoms) {
            const bool first = k < QP1;
            const int kl = first ? k : k - QP1;
            const int kk = first ? k0 + kl : k0 + Q1 + kl;
            const bool in = (first ? kl < Q1 : kl < Q2) && kk < a.n_q;
            s_fx[k] = in ? a.ff[(size_t)kk * a.n_types + tile.type] : 0.f;
        }
        __syncthreads();
        {
            float2 S[QP1 / 2];
#pragma unroll
            for (int m = 0; m < QP1 / 2; ++m)
                S[m] = make_float2(0.f, 0.f);
            for (int jj = 0; jj < len; ++jj) {
                const bool use = valid && s_idx[jj] != y;
                float rn, rninv, ro, roinv, dx, dy, dz;
                pair_r(py_new, s_new[jj], rn, rninv, dx, dy, dz);
                pair_r(py_old, s_old[jj], ro, roinv, dx, dy, dz);
                WideSeed pn = wide_seed(q0, dq, rn, use ? mult * rninv : 0.f, SMALL);
                WideSeed po = wide_seed(q0, dq, ro, use ? -mult * roinv : 0.f, SMALL);
                if (SMALL || !__any_sync(0xffffffffu, pn.sg < 0.f || po.sg < 0.f))
                    wide_pair2_carry<Q1, QP1 / 2, false>(pn, po, S);
                else
                    wide_pair2_carry<Q1, QP1 / 2, true>(pn, po, S);
                if constexpr (Q2 > 0) {
                    float2 *st = &u_st[(size_t)jj * 5 * kBlockAtoms + tid];
                    st[0] = pn.s;
                    st[kBlockAtoms] = pn.d;
                    st[2 * kBlockAtoms] = po.s;
                    st[3 * kBlockAtoms] = po.d;
                    st[4 * kBlockAtoms] =
                        make_float2(pack_lam_sign(pn.l, pn.sg), pack_lam_sign(po.l, po.sg));
                }
            }
#pragma unroll
            for (int c = 0; c < NR1; ++c) {
                const float v = warp_sum_rows([&](int k) { return pair_at(S, 32 * c + k); },
                                              sum_buf, lane);
                acc1[c] += (double)(s_fx[32 * c + lane] * v);
            }
        }
        if constexpr (Q2 > 0) {
            float2 S[QP2 / 2];
#pragma unroll
            for (int m = 0; m < QP2 / 2; ++m)
                S[m] = make_float2(0.f, 0.f);
            for (int jj = 0; jj < len; ++jj) {
                const float2 *st = &u_st[(size_t)jj * 5 * kBlockAtoms + tid];
                WideSeed pn, po;
                pn.s = st[0];
                pn.d = st[kBlockAtoms];
                po.s = st[2 * kBlockAtoms];
                po.d = st[3 * kBlockAtoms];
                const float2 ls = st[4 * kBlockAtoms];
                unpack_lam_sign(ls.x, pn.l, pn.sg);
                unpack_lam_sign(ls.y, po.l, po.sg);
                if (SMALL || !__any_sync(0xffffffffu, pn.sg < 0.f || po.sg < 0.f))
                    wide_pair2_carry<Q2, QP2 / 2, false>(pn, po, S);
                else
                    wide_pair2_carry<Q2, QP2 / 2, true>(pn, po, S);
            }
#pragma unroll
            for (int c = 0; c < NR2; ++c) {
                const float v = warp_sum_rows([&](int k) { return pair_at(S, 32 * c + k); },
                                              sum_buf, lane);
                acc2[c] += (double)(s_fx[QP1 + 32 * c + lane] * v);
            }
        }
    }
    __syncthreads(); // states and summation buffers are no longer read: u_red takes their place
#pragma unroll
    for (int c = 0; c < NR1; ++c)
        u_red[warp][32 * c + lane] = acc1[c];
#pragma unroll
    for (int c = 0; c < NR2; ++c)
        u_red[warp][QP1 + 32 * c + lane] = acc2[c];
    __syncthreads();
    for (int k = tid; k < QP1 + QP2; k += kBlockAtoms) {
        const bool first = k < QP1;
        const int kl = first ? k : k - QP1;
        const int kk = first ? k0 + kl : k0 + Q1 + kl;
        if ((first ? kl >= Q1 : kl >= Q2) || kk >= a.n_q)
            continue;
        double s = 0.0;
#pragma unroll
        for (int w = 0; w < kBlockAtoms / 32; ++w)
            s += u_red[w][k];
        a.partial[(size_t)kk * a.n_blocks * n_groups + (size_t)group * a.n_blocks + blockIdx.x] =
            s * (double)a.ff[(size_t)kk * a.n_types + by.type];
    }
}

__global__ void f64_to_f32_kernel(const double *src, float *dst, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        dst[i] = (float)src[i];
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
    default: // 64 and wider: the wide kernels (launch_forward_wide)
        return cudaErrorInvalidValue;
    }
}

// Occupancy: the plain instantiations (small_theta level 2) fit in 168
// registers up to 128 q, so 3 CTAs (12 warps) share an SM and hide the seed
// latency (6 % faster than 2 CTAs with 4 pairs per step at 201 q); the signed
// ones keep 2 CTAs/SM above 64 q.  Both step 2 pairs at a time.
template <int QS>
static cudaError_t wide_launch(DebyeArgs a, int k_base, int n_slabs, bool water, cudaStream_t st,
                               bool main = false)
{
    a.k_base = k_base;
    const dim3 grid(a.n_items, n_slabs);
    if constexpr (QS >= 128) {
        // the tuned tile shape: four pairs per step in the main slabs
        if (main && a.pairs4 && !water) {
            if (a.small_theta >= 2)
                forward_wide_kernel<QS, 4, false><<<grid, kBlockAtoms, 0, st>>>(a);
            else
                forward_wide_kernel<QS, 4, true><<<grid, kBlockAtoms, 0, st>>>(a);
            count_launch();
            return cudaGetLastError();
        }
    }
    if constexpr (QS > 128) {
        // no water instantiation this wide (its per-q factor rows would spill)
        if (water)
            return cudaErrorInvalidValue;
        if (a.small_theta >= 2)
            forward_wide_kernel<QS, 2, false><<<grid, kBlockAtoms, 0, st>>>(a);
        else
            forward_wide_kernel<QS, 2, true><<<grid, kBlockAtoms, 0, st>>>(a);
        count_launch();
        return cudaGetLastError();
    } else {
        if (water && a.small_theta >= 2)
            forward_wide_water_kernel<QS, false><<<grid, kBlockAtoms, 0, st>>>(a);
        else if (water)
            forward_wide_water_kernel<QS, true><<<grid, kBlockAtoms, 0, st>>>(a);
        else if (a.small_theta >= 2)
            forward_wide_kernel<QS, 2, false><<<grid, kBlockAtoms, 0, st>>>(a);
        else
            forward_wide_kernel<QS, 2, true><<<grid, kBlockAtoms, 0, st>>>(a);
        count_launch();
        return cudaGetLastError();
    }
}

// Relative cost of one slab per pair on GB300 (CUDA-event times of single
// slabs at N = 20,000 on a compact structure, plain instantiations at 3
// CTAs/SM, in ms per 2e8 pairs): full slabs of 64, 112 and 128 q, and a slab
// 16, 32, ..., 128 q wide.  The seed of a slab costs about as much as 40
// steps, so short slabs are dear per q (the 48-q slab measured slower than
// the 64-q one, which therefore also serves remainders of 33..48 q).
static constexpr float kCostMain64 = 1.82f, kCostMain112 = 2.75f, kCostMain128 = 3.00f;
// the 192-q slab (2 CTAs/SM) on the same scale: N = 200,000, 512 q took
// 1083.7 ms as four 128-q slabs and 1001.1 ms as two 192-q slabs and a
// 128-q tail, so a 192-q slab costs (1001.1 - 1083.7 / 4) / 2 / (1083.7 / 4)
// = 1.347 128-q slabs
static constexpr float kCostMain192 = 4.04f;
static constexpr float kCostWidth[8] = {0.99f, 1.35f, 2.34f, 1.82f, 2.13f, 2.29f, 2.75f, 3.00f};

// Width (multiple of 16, <= 128) of the cheapest slab that covers len q.
static int tail_width(int len)
{
    int best = 0;
    for (int w = (len + 15) / 16; w <= 8; ++w)
        if (best == 0 || kCostWidth[w - 1] < kCostWidth[best / 16 - 1])
            best = 16 * w;
    return best;
}

static float tail_cost(int len) { return len > 0 ? kCostWidth[tail_width(len) / 16 - 1] : 0.f; }

static cudaError_t wide_tail(const DebyeArgs &a, int k0, int width, bool water, cudaStream_t st)
{
    switch (width / 16) {
    case 1:
        return wide_launch<16>(a, k0, 1, water, st);
    case 2:
        return wide_launch<32>(a, k0, 1, water, st);
    case 3:
        return wide_launch<48>(a, k0, 1, water, st);
    case 4:
        return wide_launch<64>(a, k0, 1, water, st);
    case 5:
        return wide_launch<80>(a, k0, 1, water, st);
    case 6:
        return wide_launch<96>(a, k0, 1, water, st);
    case 7:
        return wide_launch<112>(a, k0, 1, water, st);
    default:
        return wide_launch<128>(a, k0, 1, water, st);
    }
}

cudaError_t launch_forward_slab(const DebyeArgs &a, int k0, int width, cudaStream_t st)
{
    return wide_tail(a, k0, width, false, st);
}

// The cheapest of: 64-q slabs and a tail; 64-q slabs with a short remainder
// (<= 48 q) folded into the last slab; 112-q or 128-q slabs and a tail
// (q_slab >= 128); 192-q slabs and a tail of at most 128 q (q_slab >= 192).
WidePlan wide_plan(int n_q, int q_slab)
{
    WidePlan best{};
    float best_cost = 3.4e38f;
    auto consider = [&](int main, int full, int rest, float cost) {
        if (cost < best_cost) {
            best_cost = cost;
            best = WidePlan{main, full, full * main, rest, rest > 0 ? tail_width(rest) : 0};
        }
    };
    const int f64 = n_q / 64, r64 = n_q - 64 * f64;
    consider(64, f64, r64, f64 * kCostMain64 + tail_cost(r64));
    if (f64 > 0 && r64 > 0 && r64 <= 48)
        consider(64, f64 - 1, r64 + 64, (f64 - 1) * kCostMain64 + tail_cost(r64 + 64));
    if (q_slab >= 128) {
        const int f112 = n_q / 112, r112 = n_q - 112 * f112;
        consider(112, f112, r112, f112 * kCostMain112 + tail_cost(r112));
        const int f128 = n_q / 128, r128 = n_q - 128 * f128;
        consider(128, f128, r128, f128 * kCostMain128 + tail_cost(r128));
    }
    if (q_slab >= 192) {
        // one tail slab of at most 128 q follows the 192-q slabs
        const int f192 = n_q / 192, r192 = n_q - 192 * f192;
        if (f192 > 0 && r192 <= 128)
            consider(192, f192, r192, f192 * kCostMain192 + tail_cost(r192));
    }
    return best;
}

// Uniform grid: full slabs of the plan's main width, then the tail slab (a
// second launch: on `aux` when given, forked after the work queued on `st`
// and joined back into it, else on `st`).
static cudaError_t launch_forward_wide(const DebyeArgs &a, int q_slab, bool water, cudaStream_t st,
                                       const AuxStream *aux)
{
    if (a.q0_free && a.n_q > 1)
        return launch_forward_wide(past_q0(a, a.n_items), q_slab, water, st, aux);
    // q_slab 192: chains of 192-q slabs with one seed per pair and chain
    // (four pairs per step keep the slab kernels), when the items fill at
    // least 4 waves of the chain kernel (2 CTAs per SM); a small structure's
    // few items get twice the CTAs from the slab kernels (one per slab)
    if (!water && q_slab >= 192 && !a.pairs4) {
        int dev = 0, sms = 152;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
            sms = 152;
        if (a.n_items >= 8 * sms)
            return launch_forward_chain(a, st, aux);
    }
    const WidePlan p = wide_plan(a.n_q, water ? std::min(q_slab, 128) : q_slab);
    const bool split = aux && p.full > 0 && p.tail_len > 0;
    if (split) {
        cudaError_t e = cudaEventRecord(aux->fork, st);
        if (e == cudaSuccess)
            e = cudaStreamWaitEvent(aux->stream, aux->fork, 0);
        if (e != cudaSuccess)
            return e;
    }
    if (p.full > 0) {
        cudaError_t e;
        e = p.main == 64    ? wide_launch<64>(a, 0, p.full, water, st)
            : p.main == 112 ? wide_launch<112>(a, 0, p.full, water, st)
            : p.main == 192 ? wide_launch<192>(a, 0, p.full, water, st, true)
                            : wide_launch<128>(a, 0, p.full, water, st, true);
        if (e != cudaSuccess)
            return e;
    }
    if (p.tail_len == 0)
        return cudaSuccess;
    if (!split)
        return wide_tail(a, p.tail_k0, p.tail_w, water, st);
    cudaError_t e = wide_tail(a, p.tail_k0, p.tail_w, water, aux->stream);
    // the join is recorded and awaited even after a failed launch, so that
    // `st` never runs ahead of work queued on the aux stream
    const cudaError_t ej = cudaEventRecord(aux->join, aux->stream);
    const cudaError_t ew = ej == cudaSuccess ? cudaStreamWaitEvent(st, aux->join, 0) : ej;
    return e != cudaSuccess ? e : ew;
}

// Uniform grids and q_slab 64 / 128 take the wide slabs (64 to 128 q per
// seed, with or without water); otherwise full slabs of q_slab values, then
// the remainder in the smallest slab of 8 / 16 / 32 that covers it (a second
// launch on the same stream).
cudaError_t launch_forward(const DebyeArgs &a, int q_slab, bool uniform, bool water,
                           cudaStream_t st, const AuxStream *aux)
{
    if (a.n_items == 0)
        return cudaSuccess;
    if (uniform && q_slab >= 64)
        return launch_forward_wide(a, q_slab, water, st, aux);
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
    assemble_kernel<<<a.n_q + (a.apply_k + 255) / 256, 256, 0, st>>>(a);
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

// SMALL (small_theta level 2: |theta| < pi/4 for every pair before and after
// the move): the seeds skip the reduction of theta and the signed steps.
template <int Q1, int Q2>
static cudaError_t delta_chain_launch(const DeltaArgs &a, int k_base, int n_chains,
                                      cudaStream_t st)
{
    const dim3 grid(a.n_blocks, n_chains, delta_groups(a));
    constexpr size_t smem = delta_chain_smem(Q2);
    auto kfn = a.small_theta >= 2 ? delta_chain_kernel<Q1, Q2, true>
                                  : delta_chain_kernel<Q1, Q2, false>;
    if (smem > 32 * 1024) { // with the static arrays past the 48 KB default
        const cudaError_t e =
            cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess)
            return e;
    }
    kfn<<<grid, kBlockAtoms, smem, st>>>(a, k_base);
    count_launch();
    return cudaGetLastError();
}

int delta_groups(const DeltaArgs &a)
{
    return std::max(1, std::min(std::min(kDeltaGroups, a.n_mtiles), a.max_groups));
}

// One chain over the last `width` q from k0: one slab of 16..112 q (a
// multiple of 16), or 112 q and a second slab of 8..112 q (a multiple of 8).
static cudaError_t delta_chain_rest(const DeltaArgs &a, int k0, int width, cudaStream_t st)
{
    if (width > 112) {
        switch ((width - 112) / 8) {
        case 1: return delta_chain_launch<112, 8>(a, k0, 1, st);
        case 2: return delta_chain_launch<112, 16>(a, k0, 1, st);
        case 3: return delta_chain_launch<112, 24>(a, k0, 1, st);
        case 4: return delta_chain_launch<112, 32>(a, k0, 1, st);
        case 5: return delta_chain_launch<112, 40>(a, k0, 1, st);
        case 6: return delta_chain_launch<112, 48>(a, k0, 1, st);
        case 7: return delta_chain_launch<112, 56>(a, k0, 1, st);
        case 8: return delta_chain_launch<112, 64>(a, k0, 1, st);
        case 9: return delta_chain_launch<112, 72>(a, k0, 1, st);
        case 10: return delta_chain_launch<112, 80>(a, k0, 1, st);
        case 11: return delta_chain_launch<112, 88>(a, k0, 1, st);
        case 12: return delta_chain_launch<112, 96>(a, k0, 1, st);
        case 13: return delta_chain_launch<112, 104>(a, k0, 1, st);
        case 14: return delta_chain_launch<112, 112>(a, k0, 1, st);
        default:
            return cudaErrorInvalidValue;
        }
    }
    switch (width / 16) {
    case 1: return delta_chain_launch<16, 0>(a, k0, 1, st);
    case 2: return delta_chain_launch<32, 0>(a, k0, 1, st);
    case 3: return delta_chain_launch<48, 0>(a, k0, 1, st);
    case 4: return delta_chain_launch<64, 0>(a, k0, 1, st);
    case 5: return delta_chain_launch<80, 0>(a, k0, 1, st);
    case 6: return delta_chain_launch<96, 0>(a, k0, 1, st);
    case 7: return delta_chain_launch<112, 0>(a, k0, 1, st);
    default:
        return cudaErrorInvalidValue;
    }
}

// Uniform grids: chains of 224 q (two 112-q slabs, one seed per pair chain)
// from q row 0 of `a` (row 1 of the grid for a past_q0 view), then one chain
// over the rest: up to 112 q rounded up to 16, past that 112 q and the
// remainder rounded up to 8 (n_q = 201 from q = 0: the 200 q past q = 0 as a
// single 112 + 88 chain, one launch).  With full chains and a rest, the rest
// goes to the aux stream when there is one, so that its CTAs fill the last
// wave of the main launch.
static cudaError_t launch_delta_wide(const DeltaArgs &a, cudaStream_t st, const AuxStream *aux)
{
    constexpr int kSpan = 224;
    const int full = a.n_q / kSpan, rest = a.n_q - full * kSpan;
    const int rest_w = rest <= 112 ? (rest + 15) / 16 * 16 : 112 + (rest - 112 + 7) / 8 * 8;
    const bool split = aux && full > 0 && rest > 0;
    if (split) {
        cudaError_t e = cudaEventRecord(aux->fork, st);
        if (e == cudaSuccess)
            e = cudaStreamWaitEvent(aux->stream, aux->fork, 0);
        if (e != cudaSuccess)
            return e;
    }
    if (full > 0) {
        const cudaError_t e = delta_chain_launch<112, 112>(a, 0, full, st);
        if (e != cudaSuccess)
            return e;
    }
    if (rest == 0)
        return cudaSuccess;
    if (!split)
        return delta_chain_rest(a, full * kSpan, rest_w, st);
    cudaError_t e = delta_chain_rest(a, full * kSpan, rest_w, aux->stream);
    // joined even after a failed launch, so that `st` never runs ahead of
    // work queued on the aux stream
    const cudaError_t ej = cudaEventRecord(aux->join, aux->stream);
    const cudaError_t ew = ej == cudaSuccess ? cudaStreamWaitEvent(st, aux->join, 0) : ej;
    return e != cudaSuccess ? e : ew;
}

int delta_parts(const DeltaArgs &a, int q_slab, bool uniform)
{
    return (uniform && q_slab >= 64) ? a.n_blocks * delta_groups(a) : a.n_blocks;
}

cudaError_t launch_delta(const DeltaArgs &a, int q_slab, bool uniform, cudaStream_t st,
                         const AuxStream *aux)
{
    if (a.n_blocks == 0 || a.k == 0)
        return cudaSuccess;
    if (uniform && q_slab >= 64)
        return launch_delta_wide(a.q0_free && a.n_q > 1 ? past_q0(a, a.n_blocks * delta_groups(a)) : a,
                                 st, aux);
    switch (q_slab > 32 ? 32 : q_slab) { // two chains per pair: at most 32 q per slab
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

cudaError_t launch_f64_to_f32(const double *src, float *dst, int n, cudaStream_t st)
{
    if (n == 0)
        return cudaSuccess;
    f64_to_f32_kernel<<<(n + 255) / 256, 256, 0, st>>>(src, dst, n);
    count_launch();
    return cudaGetLastError();
}

} // namespace rsx
