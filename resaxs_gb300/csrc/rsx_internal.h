// Internal declarations shared by the CUDA kernels and the C++ host layer of
// librsx.  Not part of the public C ABI (include/rsx.h).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace rsx {

constexpr int kMaxTypes = 32;    // factor-table columns a kernel holds in shared memory
constexpr int kBlockAtoms = 128; // bodies per block tile = threads per CTA

// A block tile: `len` (<= kBlockAtoms) consecutive bodies of one type in the
// type-sorted order, starting at `start`.
struct BlockDesc {
    int start, len, type, pad;
};

// One unit of pair work: I-block `bi` against J-blocks [bj_begin, bj_end),
// all of one type, with bj_begin >= bi (upper triangle of block pairs).
struct PairItem {
    int bi, bj_begin, bj_end, pad;
};

// How small the step angle theta = dq r is guaranteed to be for every pair
// of a uniform grid with step dq over bodies whose bounding-box diagonal is
// `diag` (an upper bound of every pair distance):
//   2: |theta| <= 0.7 < pi/4 (the paired-step seeds of the forward skip the
//      range reduction, and every pair takes the unsigned form);
//   1: |theta / 2| <= 0.7 (the half-angle seeds of the adjoint skip it);
//   0: neither (or not a uniform grid).
inline int theta_level(bool uniform, double dq, double diag)
{
    if (!uniform || !(diag >= 0.0) || !(diag < 1e30))
        return 0;
    const double t = (dq < 0.0 ? -dq : dq) * diag * 1.0001;
    return t <= 0.7 ? 2 : (t <= 1.4 ? 1 : 0);
}

// Arguments of the Debye pair kernels (forward and adjoint).
struct DebyeArgs {
    const float4 *pos;       // bodies in type-sorted order, .w = type bits
    const float *rsasa;      // per sorted body, nullptr without water
    const float *ff;         // [n_q][n_types] factor table
    const float *q;          // [n_q]
    const BlockDesc *blocks; // [n_blocks]
    const PairItem *items;   // [n_items]
    double *partial;         // [n_q][n_items] per-item cross sums (forward)
    int n, n_q, n_types, n_items;
    int k_base;              // first q index of the launch (set by the launcher)
    float dq;                // uniform q step (rotation path)
    int small_theta;         // theta_level() of the launch's bodies
    int pairs4;              // 1: the wide main slabs step 4 pairs at a time (else 2)
    float water_weight;      // w (water path)
    int water_index;         // column of the water factor
    int q0_free;             // host side: a uniform grid with q[0] == 0, q[1] == dq (past_q0)
    // adjoint
    const float *lambda;     // [n_q] dL/dI(q)
    double *grad;            // [n][3] sorted-order FP64 gradient accumulators
    // adjoint through tabulated pair functions: [member][n_types * n_types]
    // [adj_nodes] nodes (A, h A', B, h B') at r = b * h, b = 0 .. adj_nodes - 1,
    // with water four per node ([adj_nodes][4]: the factor products f_i f_j,
    // f_w f_j, f_w f_i, f_w^2 that rsasa weights 1, rs_i, rs_j, rs_i rs_j);
    // h and 1/h are adj_h / adj_inv_h, or adj_geom[0] / [1] when adj_geom is set
    // (a device copy, for captured graphs whose step changes between replays)
    const float4 *adj_tab;
    int adj_nodes;
    float adj_h, adj_inv_h;
    const float *adj_geom;
};

// Per-q constants needed to assemble I(q) from the cross sums.
struct AssembleArgs {
    const double *partial;   // [n_q][n_parts]
    const float *ff;         // [n_q][n_types]
    const float *q;
    const int *type_count;   // [n_types]
    const double *rsasa_sum; // [n_types] sum of rsasa per type (water)
    double rsasa_sq_sum;     // sum of rsasa^2 (water)
    double rsasa_total;      // sum of rsasa (water)
    int n_q, n_types, n_parts;
    float water_weight;
    int water_index;
    int has_water;
    double *iq64;            // [n_q] result (or accumulation target)
    float *iq32;             // [n_q] FP32 copy of iq64
    int accumulate;          // 1: iq64 += 2*cross/q (incremental mode, no self terms)
    // incremental mode: the moved bodies take their new positions in the same
    // launch (extra CTAs past the n_q assembling ones), pos[idx[m]] = new[m]
    float4 *apply_pos;
    const float4 *apply_new;
    const int *apply_idx;
    int apply_k;
};

// Moved-set description for the incremental kernel.
struct DeltaArgs {
    const float4 *pos_old;   // [n] sorted positions before the move
    const float4 *moved_new; // [k] new positions of the moved bodies, grouped by type
    const int *moved_idx;    // [k] sorted index of each moved body
    const BlockDesc *blocks; // [n_blocks] static-side blocks
    const BlockDesc *mtiles; // [n_mtiles] moved-list tiles (start/len into the list, type)
    const float *ff, *q;
    double *partial;         // [n_q][n_blocks]
    int n, k, n_q, n_types, n_blocks, n_mtiles;
    int max_groups;          // cap on the moved-list groups (partial holds n_blocks * groups rows)
    float dq;
    int small_theta;         // theta_level() of the bodies before and after the move
    int q0_free;             // host side: a uniform grid with q[0] == 0, q[1] == dq (past_q0)
};

constexpr int kDeltaGroups = 16; // moved-list groups of the wide delta kernel (at most)
constexpr int kDeltaTile = 8;   // moved bodies per tile of the wide delta kernel

// I(0) = (sum of the factors)^2 needs no pair sum: the assembly kernels take
// it from the type counts, and an incremental step leaves it unchanged.  So
// the wide uniform launches over a grid that starts at q = 0 run on q[1..]
// only, through a view of the q, factor and partial arrays one row in (the
// kernels index them by q row and never see the shift).  Partial row 0 is
// then not written; every reader skips it at q = 0.
template <class Args>
inline Args past_q0(const Args &a, int parts)
{
    Args v = a;
    v.q += 1;
    v.ff += a.n_types;
    v.partial += parts;
    v.n_q -= 1;
    v.q0_free = 0;
    return v;
}

// launchers (debye_kernels.cu, adjoint_kernels.cu); all asynchronous on `st`
// Slab plan of the wide uniform forward: `full` slabs of `main` q from q 0,
// then one tail slab covering [tail_k0, tail_k0 + tail_len) with a kernel
// `tail_w` q wide (tail_len 0: none).  q_slab 64 restricts the plan to 64-q
// main slabs; 128 also allows 112- and 128-q slabs.
struct WidePlan {
    int main, full, tail_k0, tail_len, tail_w;
};
WidePlan wide_plan(int n_q, int q_slab);

// A second stream for the tail slab of a wide forward, so that it runs
// beside the main slabs and fills their last wave; `fork` and `join` are
// events (timing disabled) owned with the stream.
struct AuxStream {
    cudaStream_t stream;
    cudaEvent_t fork, join;
};
cudaError_t launch_forward(const DebyeArgs &a, int q_slab, bool uniform, bool water,
                           cudaStream_t st, const AuxStream *aux = nullptr);
// Chained forward: 192-q main slabs, at most two per chain (the recurrence
// runs at most 192 paired steps per seed; at 200,000 bodies and 512 q, chains
// of three slabs left 3e-6 of error 250 paired steps after the seed), J
// sub-tiles of 32 bodies whose recurrence states wait in shared memory
// between slabs.
constexpr int kChainMain = 192;
constexpr int kChainMaxMain = 2;
constexpr int kChainPairs = 32;
// dynamic shared memory of a chain CTA: the states, then the per-warp FP64
// lane accumulators of q_slots q
__host__ __device__ constexpr size_t chain_state_bytes()
{
    return (sizeof(float2) * 2 + sizeof(float)) * kChainPairs * kBlockAtoms;
}
__host__ __device__ constexpr size_t chain_smem_bytes(int q_slots)
{
    return chain_state_bytes() + sizeof(double) * (kBlockAtoms / 32) * (size_t)q_slots;
}
// Chained forward on uniform grids without water (chain_kernels.cu): `full`
// chains of two 192-q slabs from q 0, then (rest) one chain from rest_k0 of
// rest_main 192-q slabs and a rest_tail-q tail (8, or a multiple of 16; 0
// for none); each pair is seeded once per chain.
struct ChainPlan {
    int full, rest_k0, rest_main, rest_tail;
    bool rest;
};
ChainPlan chain_plan(int n_q);
// One wide slab of `width` q (8..128: 16 or wider in steps of 16, a width of
// 8 runs as 16) from k0, no water.
cudaError_t launch_forward_slab(const DebyeArgs &a, int k0, int width, cudaStream_t st);
cudaError_t launch_forward_chain(const DebyeArgs &a, cudaStream_t st, const AuxStream *aux);
cudaError_t launch_assemble(const AssembleArgs &a, cudaStream_t st);
// adjoint through tabulated pair functions: builds the tables of the present
// type pairs into `tab` ([n_types^2][adj_nodes] float4, times 4 with water),
// then the pair pass
cudaError_t launch_adjoint_table(const DebyeArgs &a, float4 *tab, unsigned type_mask, bool water,
                                 cudaStream_t st);
// forward through the gridded pair-distance distribution (grid_kernels.cu):
// non-uniform q grids; writes partial[k][0] (one part per q) from FP64
// histograms ([n_types^2][hists][2][nodes] at the start of `hist`, followed
// by the g tables) on nodes r = b h
int forward_grid_hists(bool water);
int forward_grid_max_nodes(bool water);
// doubles the buffer of launch_forward_grid holds (histograms, then the
// [2][n_q][nodes] tables of g and h g')
size_t forward_grid_doubles(int n_types, int n_q, int nodes, bool water);
cudaError_t launch_forward_grid(const DebyeArgs &a, double *hist, int nodes, float h,
                                unsigned type_mask, bool water, cudaStream_t st);
// the tables alone, for `n_members` members (batched passes)
cudaError_t launch_adjoint_tables(const DebyeArgs &a, float4 *tab, unsigned type_mask,
                                  int n_members, cudaStream_t st);
cudaError_t launch_delta(const DeltaArgs &a, int q_slab, bool uniform, cudaStream_t st,
                         const AuxStream *aux = nullptr);
// partial sums per q that launch_delta writes (the assembly's n_parts)
int delta_parts(const DeltaArgs &a, int q_slab, bool uniform);
int delta_groups(const DeltaArgs &a);
cudaError_t launch_f64_to_f32(const double *src, float *dst, int n, cudaStream_t st);
cudaError_t launch_adjoint(const DebyeArgs &a, int q_slab, bool uniform, bool water,
                           cudaStream_t st);

// count of kernels this library has launched (for the benchmark's launch claim)
void count_launch(int n = 1);
unsigned long long launch_count();

} // namespace rsx
