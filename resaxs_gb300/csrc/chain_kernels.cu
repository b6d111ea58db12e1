// Forward Debye sums on a uniform q grid with one seed per pair and chain
// (sm_103a).  Written from scratch for this project.
//
// The wide slab kernels (debye_kernels.cu) seed every pair once per slab of
// at most 192 q: distance, 1/r, sin/cos(theta) and, past q = 0,
// sin/cos(q0 r), about 60 FP32 operations against 288 for the 192-q
// recurrence itself.  Here a CTA runs one work item over a chain of slabs:
// up to three 192-q main slabs and one tail slab of QT q (QT a multiple of
// 16, 0 for none).  The J side of the item is taken kChainPairs bodies at a
// time; every pair chain of such a sub-tile is seeded once, at the start of
// the chain, runs Reinsch's recurrence through the first slab, leaves its
// state (s, d of the even/odd sequences and lam with the sign of the odd
// steps) in shared memory while the slab's sums are reduced, and resumes
// from it in the next slab.  The per-thread FP32 slab sums of a sub-tile are
// reduce-scattered over the warp and added to per-lane FP64 accumulators in
// shared memory (lane L owns q index 32 c + L of every slab).  The chain of
// 288 paired steps at most is three times as long as a slab's; the tests hold
// it to the same 1e-5 of the FP64 oracle.
#include "debye_device.cuh"

#include <algorithm>

namespace rsx {

constexpr int kChainMain = 192;     // q per main slab
constexpr int kChainMaxMain = 3;    // main slabs per chain
constexpr int kChainPairs = 32;     // J bodies per sub-tile (chain states kept per thread)

// Dynamic shared memory of a chain CTA: the chain states, then the per-warp
// FP64 lane accumulators of `q_slots` q.
__host__ __device__ constexpr size_t chain_state_bytes()
{
    return (sizeof(float2) * 2 + sizeof(float)) * kChainPairs * kBlockAtoms;
}
__host__ __device__ constexpr size_t chain_smem_bytes(int q_slots)
{
    return chain_state_bytes() + sizeof(double) * (kBlockAtoms / 32) * (size_t)q_slots;
}

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

// One work item over q [k0, k0 + n_main * 192 + QT): writes
// partial[k][item_idx] = sum over the item's pairs of f_i f_j sin(q_k r)/r.
// q_slots = n_main * 192 + QT rounded up to 32 (the accumulator stride).
template <int QT, bool SIGNED>
__global__ void __launch_bounds__(kBlockAtoms, 2)
    forward_chain_kernel(const DebyeArgs a, int k_chain0, int chain_q, int n_main, int q_slots)
{
    constexpr int QM = kChainMain, QH = QM / 2, T = kChainPairs;
    static_assert(QT % 16 == 0 && QT <= QM, "tail slab");
    __shared__ float4 s_pos[kBlockAtoms];
    extern __shared__ __align__(16) unsigned char dsm[];
    float2 *st_sd = reinterpret_cast<float2 *>(dsm);                       // [T][2][128]
    float *st_l = reinterpret_cast<float *>(dsm + sizeof(float2) * 2 * T * kBlockAtoms); // [T][128]
    double *acc = reinterpret_cast<double *>(dsm + chain_state_bytes());   // [4][q_slots]

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int k0 = k_chain0 + blockIdx.y * chain_q;
    const int item_idx = blockIdx.x;
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
                        p1 = wide_seed(q0, dq, r1, u1 ? ri1 : 0.f, small_th);
                        p2 = wide_seed(q0, dq, r2, u2 ? ri2 : 0.f, small_th);
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

template <int QT>
static cudaError_t chain_launch(const DebyeArgs &a, int k_chain0, int n_chains, int n_main,
                                cudaStream_t st)
{
    const int chain_q = n_main * kChainMain + QT;
    const int q_slots = n_main * kChainMain + (QT + 31) / 32 * 32;
    const size_t smem = chain_smem_bytes(q_slots);
    auto kfn = a.small_theta >= 2 ? forward_chain_kernel<QT, false> : forward_chain_kernel<QT, true>;
    if (smem > 32 * 1024) { // with the static arrays past the 48 KB default
        const cudaError_t e =
            cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess)
            return e;
    }
    kfn<<<dim3(a.n_items, n_chains), kBlockAtoms, smem, st>>>(a, k_chain0, chain_q, n_main, q_slots);
    count_launch();
    return cudaGetLastError();
}

static cudaError_t chain_launch_tail(const DebyeArgs &a, int k_chain0, int n_chains, int n_main,
                                     int tail_w, cudaStream_t st)
{
    switch (tail_w / 16) {
    case 0: return chain_launch<0>(a, k_chain0, n_chains, n_main, st);
    case 1: return chain_launch<16>(a, k_chain0, n_chains, n_main, st);
    case 2: return chain_launch<32>(a, k_chain0, n_chains, n_main, st);
    case 3: return chain_launch<48>(a, k_chain0, n_chains, n_main, st);
    case 4: return chain_launch<64>(a, k_chain0, n_chains, n_main, st);
    case 5: return chain_launch<80>(a, k_chain0, n_chains, n_main, st);
    case 6: return chain_launch<96>(a, k_chain0, n_chains, n_main, st);
    case 7: return chain_launch<112>(a, k_chain0, n_chains, n_main, st);
    case 8: return chain_launch<128>(a, k_chain0, n_chains, n_main, st);
    case 9: return chain_launch<144>(a, k_chain0, n_chains, n_main, st);
    case 10: return chain_launch<160>(a, k_chain0, n_chains, n_main, st);
    case 11: return chain_launch<176>(a, k_chain0, n_chains, n_main, st);
    default:
        return cudaErrorInvalidValue;
    }
}

ChainPlan chain_plan(int n_q)
{
    constexpr int span = kChainMaxMain * kChainMain;
    ChainPlan p{};
    p.full = n_q / span;
    const int rest = n_q - p.full * span;
    p.rest_k0 = p.full * span;
    p.rest_main = rest / kChainMain;
    p.rest_tail = (rest - p.rest_main * kChainMain + 15) / 16 * 16;
    if (p.rest_tail == kChainMain) { // a rest of 177..191 q: one more main slab
        ++p.rest_main;
        p.rest_tail = 0;
    }
    p.rest = rest > 0;
    return p;
}

// Chains of three 192-q slabs from q 0, then one chain over the rest (its
// main slabs and a tail rounded up to 16 q); with both, the rest chain runs
// on the aux stream beside the full ones.
cudaError_t launch_forward_chain(const DebyeArgs &a, cudaStream_t st, const AuxStream *aux)
{
    if (a.n_items == 0)
        return cudaSuccess;
    const ChainPlan p = chain_plan(a.n_q);
    const bool split = aux && p.full > 0 && p.rest;
    if (split) {
        cudaError_t e = cudaEventRecord(aux->fork, st);
        if (e == cudaSuccess)
            e = cudaStreamWaitEvent(aux->stream, aux->fork, 0);
        if (e != cudaSuccess)
            return e;
    }
    if (p.full > 0) {
        const cudaError_t e = chain_launch<0>(a, 0, p.full, kChainMaxMain, st);
        if (e != cudaSuccess)
            return e;
    }
    if (!p.rest)
        return cudaSuccess;
    if (!split)
        return chain_launch_tail(a, p.rest_k0, 1, p.rest_main, p.rest_tail, st);
    cudaError_t e = chain_launch_tail(a, p.rest_k0, 1, p.rest_main, p.rest_tail, aux->stream);
    // joined even after a failed launch, so that `st` never runs ahead of
    // work queued on the aux stream
    const cudaError_t ej = cudaEventRecord(aux->join, aux->stream);
    const cudaError_t ew = ej == cudaSuccess ? cudaStreamWaitEvent(st, aux->join, 0) : ej;
    return e != cudaSuccess ? e : ew;
}

} // namespace rsx
