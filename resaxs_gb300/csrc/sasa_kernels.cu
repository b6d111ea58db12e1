// Dot-sphere SASA for sm_103a, written from scratch for this project.
//
// Semantics: the occlusion test of the reference's calc_rsasa kernel
// (resaxslib/src/rsasa_dot_spheres.cl:94-163) with every operation rounded to
// FP32 on its own (explicit __fmul_rn / __fadd_rn / __fsub_rn, so no FMA
// contraction):
//   ext_i = r_i + P;   dot = unit_k * ext_i;   sdot = dot + p_i
//   w_b = (P + r_b) * (P + r_b);  d = sdot - p_b
//   dist2 = (dx*dx + dy*dy) + dz*dz;   occluded iff (w_b - dist2) > 1e-4f
// A dot counts as accessible when no atom (the atom itself included)
// occludes it.  The occlusion is an OR over atoms, so any visiting order gives
// the same count; only atoms within r_i + r_b + 2P (+0.01 A) of atom i can
// occlude, which makes the cell-list prune exact.
//
// Mapping: one CTA of 128 threads per atom.  The CTA gathers the candidate
// neighbours from the 27 surrounding cells into a shared-memory list (in
// chunks of kNbCap), walking the atom's own cell first, then the face, edge
// and corner neighbours, so the list runs roughly nearest first.  Dots are
// then tested in two phases:
//  * every thread tests each of its dots against the first kPhaseA entries
//    (most buried dots meet an occluder there);
//  * the dots still open are taken one at a time by their warp, which tests
//    32 further neighbours per step (one per lane) until a ballot finds an
//    occluder or the list ends.
// A thread-per-dot loop over the whole list would run each warp as long as
// its slowest dot (an exposed dot scans every candidate).
#include "rsx_internal.h"
#include "rsx_sasa_internal.h"

namespace rsx {

constexpr int kSasaThreads = 128;
constexpr int kNbCap = 1024;
constexpr int kPhaseA = 96; // neighbours every thread tests per dot before the warp takes over

// The 27 cell offsets (dx, dy, dz) in order of distance: own cell, faces,
// edges, corners.
__constant__ signed char c_cell_order[27][3] = {
    {0, 0, 0},   {-1, 0, 0},  {1, 0, 0},   {0, -1, 0},  {0, 1, 0},   {0, 0, -1},  {0, 0, 1},
    {-1, -1, 0}, {-1, 1, 0},  {1, -1, 0},  {1, 1, 0},   {-1, 0, -1}, {-1, 0, 1},  {1, 0, -1},
    {1, 0, 1},   {0, -1, -1}, {0, -1, 1},  {0, 1, -1},  {0, 1, 1},   {-1, -1, -1}, {-1, -1, 1},
    {-1, 1, -1}, {-1, 1, 1},  {1, -1, -1}, {1, -1, 1},  {1, 1, -1},  {1, 1, 1}};

__device__ __forceinline__ bool occludes(float sx, float sy, float sz, float4 b)
{
    const float dx = __fsub_rn(sx, b.x);
    const float dy = __fsub_rn(sy, b.y);
    const float dz = __fsub_rn(sz, b.z);
    const float dist2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
    return __fsub_rn(b.w, dist2) > 0.0001f;
}

__global__ void __launch_bounds__(kSasaThreads) sasa_kernel(const SasaArgs a)
{
    __shared__ float4 s_nb[kNbCap]; // x, y, z, (P + r_b)^2
    __shared__ int s_count;
    __shared__ unsigned s_exposed;
    __shared__ unsigned long long s_tests;

    const int i = blockIdx.x; // sorted (cell) order
    const int tid = threadIdx.x;
    const float4 pi = a.atoms[i]; // .w = radius
    const float probe = a.probe;
    const float ext = __fadd_rn(pi.w, probe);
    const int dots_per_thread = (a.n_dots + kSasaThreads - 1) / kSasaThreads;
    unsigned occluded = 0; // bit t: dot tid + t * kSasaThreads
    for (int t = 0; t < dots_per_thread; ++t)
        if (tid + t * kSasaThreads >= a.n_dots)
            occluded |= 1u << t;
    if (tid == 0) {
        s_exposed = 0;
        s_tests = 0;
    }
    unsigned long long tests = 0;

    // cell of atom i and the candidate range
    const int cx = a.cell_of[i * 3 + 0], cy = a.cell_of[i * 3 + 1], cz = a.cell_of[i * 3 + 2];
    const float reach = pi.w + a.max_radius + 2.0f * probe + 0.01f;
    const float reach2 = reach * reach;

    // iterate the 27 cells as a flat sequence of candidate atoms, in chunks
    // that fit the shared list
    int cell_idx = 0;      // 0..26
    int cell_pos = 0;      // position inside the current cell
    bool more = true;
    while (more) {
        __syncthreads();
        if (tid == 0)
            s_count = 0;
        __syncthreads();
        // thread 0 walks the cells; the CTA filters in parallel batches
        // (all threads read the same loop state from registers computed identically)
        while (true) {
            // locate the next non-empty cell range (same on every thread)
            int begin = 0, end = 0;
            bool found = false;
            while (cell_idx < 27) {
                const int ox = c_cell_order[cell_idx][0], oy = c_cell_order[cell_idx][1],
                          oz = c_cell_order[cell_idx][2];
                const int x = cx + ox, y = cy + oy, z = cz + oz;
                if (x >= 0 && y >= 0 && z >= 0 && x < a.dims[0] && y < a.dims[1] && z < a.dims[2]) {
                    const int c = (x * a.dims[1] + y) * a.dims[2] + z;
                    begin = a.cell_start[c] + cell_pos;
                    end = a.cell_start[c + 1];
                    if (begin < end) {
                        found = true;
                        break;
                    }
                }
                ++cell_idx;
                cell_pos = 0;
            }
            if (!found) {
                more = false;
                break;
            }
            // room left in the list decides how many candidates this batch takes
            __syncthreads();
            const int room = kNbCap - s_count;
            __syncthreads();
            if (room < kSasaThreads)
                break; // list full enough: test dots, keep the walk state
            const int take = min(end - begin, kSasaThreads);
            if (tid < take) {
                const float4 b = a.atoms[begin + tid];
                const float dx = b.x - pi.x, dy = b.y - pi.y, dz = b.z - pi.z;
                if (dx * dx + dy * dy + dz * dz < reach2) {
                    const float e = __fadd_rn(probe, b.w);
                    const int slot = atomicAdd(&s_count, 1);
                    s_nb[slot] = make_float4(b.x, b.y, b.z, __fmul_rn(e, e));
                }
            }
            cell_pos += take;
            if (begin + take >= end) {
                ++cell_idx;
                cell_pos = 0;
            }
        }
        __syncthreads();
        const int n_nb = s_count;
        const int n_a = min(n_nb, kPhaseA);
        const int lane = tid & 31, warp_base = tid & ~31;
        // phase A: every thread, its own dots, the first n_a neighbours
        unsigned open = 0; // bit t: dot t still open after phase A
        for (int t = 0; t < dots_per_thread; ++t) {
            if (occluded & (1u << t))
                continue;
            const int k = tid + t * kSasaThreads;
            const float sx = __fadd_rn(__fmul_rn(a.unit[3 * k + 0], ext), pi.x);
            const float sy = __fadd_rn(__fmul_rn(a.unit[3 * k + 1], ext), pi.y);
            const float sz = __fadd_rn(__fmul_rn(a.unit[3 * k + 2], ext), pi.z);
            int n = 0;
            for (; n < n_a; ++n) {
                if (occludes(sx, sy, sz, s_nb[n])) {
                    occluded |= 1u << t;
                    ++n;
                    break;
                }
            }
            tests += (unsigned long long)n;
            if (!(occluded & (1u << t)) && n_nb > n_a)
                open |= 1u << t;
        }
        // phase B: the warp takes its open dots one at a time, 32 neighbours a step
        for (int t = 0; t < dots_per_thread; ++t) {
            unsigned pending = __ballot_sync(0xffffffffu, (open >> t) & 1u);
            while (pending) {
                const int owner = __ffs(pending) - 1;
                pending &= pending - 1;
                const int k = warp_base + owner + t * kSasaThreads;
                const float sx = __fadd_rn(__fmul_rn(a.unit[3 * k + 0], ext), pi.x);
                const float sy = __fadd_rn(__fmul_rn(a.unit[3 * k + 1], ext), pi.y);
                const float sz = __fadd_rn(__fmul_rn(a.unit[3 * k + 2], ext), pi.z);
                int tested = n_nb - n_a;
                for (int j0 = n_a; j0 < n_nb; j0 += 32) {
                    const int j = j0 + lane;
                    const bool hit = j < n_nb && occludes(sx, sy, sz, s_nb[j]);
                    const unsigned ball = __ballot_sync(0xffffffffu, hit);
                    if (ball) {
                        tested = j0 - n_a + __ffs(ball);
                        if (lane == owner)
                            occluded |= 1u << t;
                        break;
                    }
                }
                if (lane == owner)
                    tests += (unsigned long long)tested;
            }
        }
    }
    unsigned exposed = 0;
    for (int t = 0; t < dots_per_thread; ++t)
        exposed += (occluded & (1u << t)) ? 0u : 1u;
    atomicAdd(&s_exposed, exposed);
    if (a.tests)
        atomicAdd(&s_tests, tests);
    __syncthreads();
    if (tid == 0) {
        a.counts[a.orig_index[i]] = s_exposed;
        if (a.tests)
            atomicAdd(a.tests, s_tests);
    }
}

cudaError_t launch_sasa(const SasaArgs &a, cudaStream_t st)
{
    if (a.n_atoms == 0)
        return cudaSuccess;
    if (a.n_dots > kSasaThreads * 32)
        return cudaErrorInvalidValue;
    sasa_kernel<<<a.n_atoms, kSasaThreads, 0, st>>>(a);
    count_launch();
    return cudaGetLastError();
}

} // namespace rsx
