// Chained forward on a uniform q grid without water (sm_103a): one seed per
// pair and chain of up to two 192-q slabs and a tail slab.  Written from
// scratch for this project; the per-item code is forward_chain_item in
// debye_device.cuh.  The wide slab kernels (debye_kernels.cu) seed every pair
// once per slab: distance, 1/r, sin/cos(theta) and, past q = 0,
// sin/cos(q0 r), about 60 FP32 operations against 288 for the 192-q
// recurrence; a chain keeps the recurrence states of a 32-body J sub-tile in
// shared memory between slabs instead.  The chain of 192 paired steps at most
// is twice as long as a slab's; the tests hold it to the same 1e-5 of the
// FP64 oracle.
#include "debye_device.cuh"

#include <algorithm>

namespace rsx {

// One CTA per (work item, chain): the chains start at k_chain0 + y * chain_q.
template <int QT, bool SIGNED>
__global__ void __launch_bounds__(kBlockAtoms, 2)
    forward_chain_kernel(const DebyeArgs a, int k_chain0, int chain_q, int n_main, int q_slots)
{
    extern __shared__ __align__(16) unsigned char dsm[];
    // chains with a tail slab take the seeds of wide_seed_x0_first (measured
    // faster there; the same values)
    forward_chain_item<QT, SIGNED, (QT > 0)>(a, blockIdx.x, k_chain0 + blockIdx.y * chain_q,
                                             chain_q, n_main, q_slots, dsm);
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
    if (tail_w == 8)
        return chain_launch<8>(a, k_chain0, n_chains, n_main, st);
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
    // the tail in steps of 16 q, or 8 for a remainder of 1..8 q (n_q = 201
    // from q = 0: the 200 q past q = 0 make one chain of 192 + 8)
    const int left = rest - p.rest_main * kChainMain;
    p.rest_tail = left > 0 && left <= 8 ? 8 : (left + 15) / 16 * 16;
    if (p.rest_tail == kChainMain) { // a rest of 177..191 q: one more main slab
        ++p.rest_main;
        p.rest_tail = 0;
    }
    p.rest = rest > 0;
    return p;
}

// Chains of two 192-q slabs from q row 0 of `a` (row 1 of the grid for a
// past_q0 view), then one chain over the rest (its main slabs and a tail of
// chain_plan's width); with both, the rest chain runs on the aux stream
// beside the full ones.
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
    // a rest of one tail slab only: the slab kernel (a chain pays its
    // sub-tile reductions for nothing when no slab follows)
    auto rest = [&](cudaStream_t s) {
        return p.rest_main == 0 && p.rest_tail <= 128
                   ? launch_forward_slab(a, p.rest_k0, std::max(16, p.rest_tail), s)
                   : chain_launch_tail(a, p.rest_k0, 1, p.rest_main, p.rest_tail, s);
    };
    if (!split)
        return rest(st);
    cudaError_t e = rest(aux->stream);
    // joined even after a failed launch, so that `st` never runs ahead of
    // work queued on the aux stream
    const cudaError_t ej = cudaEventRecord(aux->join, aux->stream);
    const cudaError_t ew = ej == cudaSuccess ? cudaStreamWaitEvent(st, aux->join, 0) : ej;
    return e != cudaSuccess ? e : ew;
}

} // namespace rsx
