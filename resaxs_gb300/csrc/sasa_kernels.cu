// Dot-sphere SASA for sm_103a, written from scratch for this project.
//
// Semantics: the occlusion test of the reference's calc_rsasa kernel
// (resaxslib/src/rsasa_dot_spheres.cl:94-163) and of its CPU algorithm
// (resaxslib/src/rsasa_cpu_alg.cpp:62-69), every operation rounded to FP32
// on its own (no FMA contraction):
//   dot = d + p_i        d = unit_k * (r_i + P) (unit form) or the caller's
//                        pre-scaled dot of atom i's type (typed form)
//   w_b = (P + r_b) * (P + r_b);   dist2 = (dx*dx + dy*dy) + dz*dz
//   occluded iff (w_b - dist2) > 1e-4f;  a dot whose x is not finite is padding
// A dot is accessible when no atom (the atom itself included) occludes it.
// The test is an OR over atoms, so any visiting order gives the same count.
//
// Cell list (built here from the caller-order atoms): a cell is at least as
// wide as the largest reach |d| + P + r_b of any occluder, so the 27 cells
// around an atom hold every atom that can occlude one of its dots.  Cells
// are binned with atomics (the order inside a cell varies between calls;
// the counts do not).
//
// Occlusion pass, one warp per atom:
//  * the warp reads the 9 rows of 3 cells along z around the atom (each row
//    is one contiguous range of the cell-ordered atoms) and keeps the atoms
//    within reach in a shared-memory list (chunks of kListCap);
//  * the list is sorted by distance band (8 bands; nearest atoms occlude
//    most dots, so most dots meet their occluder in the first few
//    candidates) into pairs for the FP32x2 units: (x0, x1, y0, y1),
//    (z0, z1, -w0, -w1);
//  * the atom's dots come in groups of 32 that are compact on the sphere
//    (ordered so by the host), one dot per lane.  All lanes test the same
//    candidates (shared-memory broadcast), four per step, two per FP32x2
//    instruction; neighbouring dots tend to close on the same occluder, so
//    the lanes of a group finish close together;
//  * when a group is down to a few open dots with many candidates left, the
//    warp takes those dots one at a time and tests 64 candidates per step
//    (a pair per lane).
// The subtraction s - b is formed as b + (-s) and w - dist2 as
// -(dist2 + (-w)): negation is exact and round-to-nearest is symmetric, so
// every value has the bits of the reference's expression.
#include "rsx_internal.h"
#include "rsx_sasa_internal.h"

namespace rsx {

constexpr int kSasaWarps = 4;      // warps (atoms) per CTA
constexpr int kListCap = 192;      // candidates per warp in shared memory at a time (<= 8 rows)
constexpr unsigned kFull = 0xffffffffu;

// Cell coordinates in FP64: atoms closer than one cell width never land two
// cells apart, whatever the grid's extent.
__device__ __forceinline__ void cell_coords(float x, float y, float z, const float lo[3],
                                            double inv_cell, const int dims[3], int c[3])
{
    const float v[3] = {x, y, z};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        int k = (int)floor(((double)v[a] - (double)lo[a]) * inv_cell);
        c[a] = min(max(k, 0), dims[a] - 1);
    }
}

// ---- geometry of the call ---------------------------------------------------

// Ordered keys of floats: key(a) < key(b) iff a < b (for non-NaN values), so
// atomicMax / atomicMin on the keys reduce floats.
__device__ __forceinline__ unsigned float_key(float f)
{
    const unsigned b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float key_float(unsigned k)
{
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

// Checks of every atom (finite position; radius >= 0 and finite, or type
// below n_types) and the reductions the grid needs: bounding box, largest
// |coordinate|, largest radius (unit form) and the types present (typed
// form).  geom is zero on entry; box minima are kept as complemented keys.
__global__ void __launch_bounds__(256) sasa_geom_kernel(const SasaCellArgs c)
{
    __shared__ unsigned s_present[kSasaMaxTypes / 32];
    const int tid = threadIdx.x, lane = tid & 31;
    if (tid < kSasaMaxTypes / 32)
        s_present[tid] = 0u;
    __syncthreads();
    unsigned lo_k[3] = {0u, 0u, 0u}, hi_k[3] = {0u, 0u, 0u}, amax_k = 0u, rmax_k = 0u, bad = 0u;
    for (int i = blockIdx.x * blockDim.x + tid; i < c.n_atoms; i += gridDim.x * blockDim.x) {
        const float4 p = c.atoms_in[i];
        const float v[3] = {p.x, p.y, p.z};
        float am = 0.f;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const float av = fabsf(v[a]);
            if (!(av <= 3.402823466e38f)) {
                bad = 1u;
                continue;
            }
            lo_k[a] = max(lo_k[a], ~float_key(v[a]));
            hi_k[a] = max(hi_k[a], float_key(v[a]));
            am = fmaxf(am, av);
        }
        amax_k = max(amax_k, __float_as_uint(am));
        if (c.radii_in) {
            const float r = c.radii_in[i];
            if (!(r >= 0.f && r <= 3.402823466e38f))
                bad = 1u;
            else
                rmax_k = max(rmax_k, __float_as_uint(r));
        } else {
            const unsigned t = __float_as_uint(p.w);
            if (t >= (unsigned)c.n_types)
                bad = 1u;
            else
                atomicOr(&s_present[t >> 5], 1u << (t & 31));
        }
    }
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            lo_k[a] = max(lo_k[a], __shfl_xor_sync(kFull, lo_k[a], o));
            hi_k[a] = max(hi_k[a], __shfl_xor_sync(kFull, hi_k[a], o));
        }
        amax_k = max(amax_k, __shfl_xor_sync(kFull, amax_k, o));
        rmax_k = max(rmax_k, __shfl_xor_sync(kFull, rmax_k, o));
        bad |= __shfl_xor_sync(kFull, bad, o);
    }
    SasaGeom *g = c.geom;
    if (lane == 0) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            atomicMax(&g->lo_key[a], lo_k[a]);
            atomicMax(&g->hi_key[a], hi_k[a]);
        }
        atomicMax(&g->amax_key, amax_k);
        atomicMax(&g->rmax_key, rmax_k);
        if (bad)
            atomicOr(&g->bad, 1u);
    }
    __syncthreads();
    if (tid < kSasaMaxTypes / 32 && s_present[tid])
        atomicOr(&g->present[tid], s_present[tid]);
}

// The cell grid from the reductions (one thread): a cell is at least as wide
// as the largest reach |d| + P + r_b (plus a margin for the rounding of the
// dot position), widened by 1.5 until the grid has at most 4 n + 4096 cells.
__global__ void sasa_plan_kernel(const SasaCellArgs c)
{
    if (threadIdx.x != 0)
        return;
    SasaGeom *g = c.geom;
    if (g->bad)
        return;
    float lo[3], hi[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        lo[a] = key_float(~g->lo_key[a]);
        hi[a] = key_float(g->hi_key[a]);
    }
    const float amax = __uint_as_float(g->amax_key);
    float rmax = __uint_as_float(g->rmax_key), dmax = 0.f;
    if (!c.radii_in) {
        rmax = 0.f;
        for (int t = 0; t < c.n_types; ++t)
            if ((g->present[t >> 5] >> (t & 31)) & 1u) {
                rmax = fmaxf(rmax, c.type_radius[t]);
                dmax = fmaxf(dmax, c.dot_reach[t]);
            }
    } else {
        dmax = (rmax + c.probe) * c.unit_reach;
    }
    const float margin = 0.01f + 8e-6f * amax;
    double cell = ((double)dmax * 1.000001 + c.probe + rmax + margin) * 1.001 + 1e-3;
    double d[3];
    for (;;) {
        double total = 1.0;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            d[a] = floor(((double)hi[a] - (double)lo[a]) / cell) + 1.0;
            total *= d[a];
        }
        if (total <= 4.0 * c.n_atoms + 4096.0)
            break;
        cell *= 1.5; // sparse, wide boxes: fewer, larger cells (still exact)
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        g->lo[a] = lo[a];
        g->dims[a] = (int)d[a];
    }
    g->n_cells = (int)d[0] * (int)d[1] * (int)d[2];
    g->margin = margin;
    g->inv_cell = 1.0 / cell;
}

// ---- cell list --------------------------------------------------------------

__global__ void sasa_bin_kernel(const SasaCellArgs c)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const SasaGeom *g = c.geom;
    if (i >= c.n_atoms || g->bad)
        return;
    const float4 p = c.atoms_in[i];
    int k[3];
    cell_coords(p.x, p.y, p.z, g->lo, g->inv_cell, g->dims, k);
    const int cid = (k[0] * g->dims[1] + k[1]) * g->dims[2] + k[2];
    c.cell_of[i] = cid;
    c.rank_of[i] = atomicAdd(&c.cell_count[cid], 1);
}

// Exclusive prefix sum of the cell counts by one CTA (cells number at most
// 4 n + 4096), 4 cells per thread per tile.
__global__ void __launch_bounds__(1024) sasa_scan_kernel(const int *count, int *start,
                                                          const SasaGeom *g)
{
    __shared__ int s_warp[32];
    __shared__ int s_carry;
    if (g->bad)
        return; // the whole CTA leaves before its first barrier
    const int n = g->n_cells;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0)
        s_carry = 0;
    __syncthreads();
    for (int base = 0; base < n; base += 4 * 1024) {
        int v[4], sum = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int idx = base + threadIdx.x * 4 + k;
            v[k] = idx < n ? count[idx] : 0;
            sum += v[k];
        }
        int x = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(kFull, x, o);
            if (lane >= o)
                x += y;
        }
        if (lane == 31)
            s_warp[warp] = x;
        __syncthreads();
        if (warp == 0) {
            int w = s_warp[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(kFull, w, o);
                if (lane >= o)
                    w += y;
            }
            s_warp[lane] = w;
        }
        __syncthreads();
        int excl = s_carry + (warp ? s_warp[warp - 1] : 0) + x - sum;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int idx = base + threadIdx.x * 4 + k;
            if (idx < n)
                start[idx] = excl;
            excl += v[k];
        }
        __syncthreads();
        if (threadIdx.x == 1023)
            s_carry = excl;
        __syncthreads();
    }
    if (threadIdx.x == 0)
        start[n] = s_carry;
}

__global__ void sasa_scatter_kernel(const SasaCellArgs c)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n_atoms || c.geom->bad)
        return;
    const float4 p = c.atoms_in[i];
    const int s = c.cell_start[c.cell_of[i]] + c.rank_of[i];
    // (types were checked by sasa_geom_kernel: a bad one stops the call)
    float r;
    if (c.radii_in) {
        r = c.radii_in[i];
    } else {
        const int t = (int)__float_as_uint(p.w);
        r = c.type_radius[t];
        c.type_of[s] = t;
    }
    c.atoms[s] = make_float4(p.x, p.y, p.z, r);
    c.orig_index[s] = i;
    c.cell_sorted[s] = c.cell_of[i];
}

cudaError_t launch_sasa_cells(const SasaCellArgs &c, cudaStream_t st)
{
    if (c.n_atoms == 0)
        return cudaSuccess;
    if ((long long)c.cells_cap < 4LL * c.n_atoms + 4097)
        return cudaErrorInvalidValue;
    cudaError_t e = cudaMemsetAsync(c.geom, 0, sizeof(SasaGeom), st);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(c.cell_count, 0, sizeof(int) * (size_t)c.cells_cap, st);
    if (e != cudaSuccess)
        return e;
    const int blocks = (c.n_atoms + 255) / 256;
    sasa_geom_kernel<<<std::min(blocks, 1024), 256, 0, st>>>(c);
    sasa_plan_kernel<<<1, 32, 0, st>>>(c);
    sasa_bin_kernel<<<blocks, 256, 0, st>>>(c);
    sasa_scan_kernel<<<1, 1024, 0, st>>>(c.cell_count, c.cell_start, c.geom);
    sasa_scatter_kernel<<<blocks, 256, 0, st>>>(c);
    count_launch(5);
    return cudaGetLastError();
}

// ---- occlusion pass ---------------------------------------------------------

constexpr int kBuckets = 8;        // distance bands of the candidate sort
constexpr int kRows = kListCap / 32;

// Two candidates against one dot: bit 0 / bit 1 set when candidate 0 / 1 of
// the pair occludes it.  A = (x0, x1, y0, y1), B = (z0, z1, -w0, -w1); n* are
// the dot's negated coordinates in both halves.
__device__ __forceinline__ unsigned occludes_pair(float2 nx, float2 ny, float2 nz, float4 A,
                                                  float4 B)
{
    const float2 dx = __fadd2_rn(make_float2(A.x, A.y), nx);
    const float2 dy = __fadd2_rn(make_float2(A.z, A.w), ny);
    const float2 dz = __fadd2_rn(make_float2(B.x, B.y), nz);
    const float2 d2 =
        __fadd2_rn(__fadd2_rn(__fmul2_rn(dx, dx), __fmul2_rn(dy, dy)), __fmul2_rn(dz, dz));
    const float2 e = __fadd2_rn(d2, make_float2(B.z, B.w)); // dist2 - w = -(w - dist2)
    return (e.x < -1e-4f ? 1u : 0u) | (e.y < -1e-4f ? 2u : 0u);
}

// Dot g * 32 + lane of the atom at p (cell order) as an absolute position.
__device__ __forceinline__ float3 dot_position(const SasaArgs &a, int group, int lane, float4 p,
                                               float ext)
{
    const float4 d = a.dots[group * 32 + lane];
    if (a.typed)
        return make_float3(__fadd_rn(d.x, p.x), __fadd_rn(d.y, p.y), __fadd_rn(d.z, p.z));
    return make_float3(__fadd_rn(__fmul_rn(d.x, ext), p.x), __fadd_rn(__fmul_rn(d.y, ext), p.y),
                       __fadd_rn(__fmul_rn(d.z, ext), p.z));
}

// Tests every open dot of the atom against the n_pairs candidate pairs of the
// warp's list (pair j: pairs[2j] = A, pairs[2j + 1] = B); updates the
// per-group open masks.  A dot whose x is not finite never opens.
__device__ void test_list(const SasaArgs &a, const float4 *pairs, int n_pairs, int n_cand,
                          unsigned *s_open, int g0, int ng, float4 p, float ext, int lane,
                          unsigned long long &tests_out)
{
    unsigned tests = 0; // < 4096 dots x kListCap candidates per call
    for (int g = 0; g < ng; ++g) {
        const unsigned open_m = s_open[g];
        if (open_m == 0)
            continue;
        const float3 s = dot_position(a, g0 + g, lane, p, ext);
        bool open = ((open_m >> lane) & 1u) && isfinite(s.x);
        const float2 nx = make_float2(-s.x, -s.x), ny = make_float2(-s.y, -s.y),
                     nz = make_float2(-s.z, -s.z);
        // (handing the last open dots to the whole warp, 64 candidates per
        // step, measured 8-10 % slower on compact and on spread structures:
        // the groups run on together until their last dot closes)
        int q = 0; // candidate pair
        while (q < n_pairs) {
            if (__ballot_sync(kFull, open) == 0)
                break;
            const unsigned h =
                occludes_pair(nx, ny, nz, pairs[2 * q], pairs[2 * q + 1]) |
                (occludes_pair(nx, ny, nz, pairs[2 * q + 2], pairs[2 * q + 3]) << 2);
            if (open && h) {
                open = false;
                tests += (unsigned)(2 * q + __ffs(h));
            }
            q += 2;
        }
        if (open)
            tests += (unsigned)n_cand;
        const unsigned m = __ballot_sync(kFull, open);
        if (lane == 0)
            s_open[g] = m;
        __syncwarp();
    }
    tests_out += tests;
}

// Sorts the n staged candidates of the warp's list (list[q] = x, y, z, -w;
// band[q] = distance band) by band, stable, into the pair layout in place,
// and pads the pairs to a multiple of 4 candidates that never occlude.
// Returns the number of pairs.
__device__ int sort_into_pairs(float4 *list, unsigned char *band, int *s_count, int n, int lane)
{
    float4 v[kRows];
    int b[kRows];
#pragma unroll
    for (int r = 0; r < kRows; ++r) {
        const int q = r * 32 + lane;
        b[r] = kBuckets; // no candidate
        v[r] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (q < n) {
            v[r] = list[q];
            b[r] = band[q];
        }
    }
    if (lane < kBuckets)
        s_count[lane] = 0;
    __syncwarp();
    const unsigned lt = (1u << lane) - 1u;
#pragma unroll
    for (int r = 0; r < kRows; ++r) {
        if (r * 32 >= n)
            break;
        const unsigned m = __match_any_sync(kFull, b[r]);
        if (b[r] < kBuckets && (m & lt) == 0u)
            s_count[b[r]] += __popc(m);
        __syncwarp();
    }
    // exclusive prefix over the bands (lanes 0..7)
    int c = lane < kBuckets ? s_count[lane] : 0;
    int x = c;
#pragma unroll
    for (int o = 1; o < kBuckets; o <<= 1) {
        const int y = __shfl_up_sync(kFull, x, o);
        if (lane >= o)
            x += y;
    }
    __syncwarp();
    if (lane < kBuckets)
        s_count[lane] = x - c;
    __syncwarp();
    float *f = reinterpret_cast<float *>(list);
#pragma unroll
    for (int r = 0; r < kRows; ++r) {
        if (r * 32 >= n)
            break;
        const unsigned m = __match_any_sync(kFull, b[r]);
        if (b[r] < kBuckets) {
            const int pos = s_count[b[r]] + __popc(m & lt);
            const int base = 8 * (pos >> 1) + (pos & 1);
            f[base] = v[r].x;
            f[base + 2] = v[r].y;
            f[base + 4] = v[r].z;
            f[base + 6] = v[r].w;
        }
        __syncwarp();
        if (b[r] < kBuckets && (m & lt) == 0u)
            s_count[b[r]] += __popc(m);
        __syncwarp();
    }
    const int padded = (n + 3) & ~3;
    if (lane < padded - n) {
        const int k = n + lane;
        f[8 * (k >> 1) + (k & 1)] = __int_as_float(0x7fc00000); // x = NaN: never occludes
    }
    __syncwarp();
    return padded >> 1;
}

__global__ void __launch_bounds__(kSasaWarps * 32, 8) sasa_kernel(const SasaArgs a)
{
    __shared__ float4 s_list[kSasaWarps][kListCap]; // staged candidates, then pairs
    __shared__ unsigned char s_band[kSasaWarps][kListCap];
    __shared__ int s_count[kSasaWarps][kBuckets];
    __shared__ unsigned s_open[kSasaWarps][kSasaMaxGroups];

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int i = blockIdx.x * kSasaWarps + warp; // cell order
    const SasaGeom *geom = a.geom;
    if (i >= a.n_atoms || geom->bad)
        return; // the whole warp leaves; no CTA-wide barrier follows
    const int dims[3] = {geom->dims[0], geom->dims[1], geom->dims[2]};
    float4 *list = s_list[warp];
    unsigned char *band = s_band[warp];
    unsigned *open = s_open[warp];

    const float4 p = a.atoms[i]; // .w = radius
    const int t = a.typed ? a.type_of[i] : 0;
    const int g0 = a.group_base[t], ng = a.group_count[t];
    const float ext = __fadd_rn(p.w, a.probe);
    // an occluder b of a dot of this atom lies within |d| + P + r_b of it
    const float dot_reach = a.typed ? a.dot_reach[t] : ext * a.unit_reach;
    const float reach = dot_reach * 1.000001f + a.probe + geom->margin;
    for (int g = lane; g < ng; g += 32)
        open[g] = kFull; // narrowed to the valid dots by the first test_list
    __syncwarp();

    // the 9 rows of 3 cells along z around the atom's cell (contiguous in
    // the cell-ordered atoms: z is the fastest cell coordinate)
    int cc[3];
    {
        const int cid = a.cell_id[i]; // (x * dims1 + y) * dims2 + z
        cc[2] = cid % dims[2];
        cc[1] = (cid / dims[2]) % dims[1];
        cc[0] = cid / (dims[2] * dims[1]);
    }
    const int z0 = max(cc[2] - 1, 0), z1 = min(cc[2] + 1, dims[2] - 1);
    int row = 0, pos = 0, n_list = 0;
    bool walk_done = false;
    unsigned long long tests = 0;
    const unsigned lt_mask = (1u << lane) - 1u;
    while (true) {
        // gather until the list cannot take another 32 and the atom itself
        while (!walk_done && n_list < kListCap - 32) {
            int beg = 0, end = 0;
            while (row < 9) {
                const int x = cc[0] + row / 3 - 1, y = cc[1] + row % 3 - 1;
                if (x >= 0 && y >= 0 && x < dims[0] && y < dims[1]) {
                    const int c = (x * dims[1] + y) * dims[2];
                    beg = a.cell_start[c + z0] + pos;
                    end = a.cell_start[c + z1 + 1];
                    if (beg < end)
                        break;
                }
                ++row;
                pos = 0;
            }
            if (row >= 9) {
                walk_done = true;
                break;
            }
            const int j = beg + lane;
            bool keep = false;
            float4 b = make_float4(0.f, 0.f, 0.f, 0.f);
            float ratio = 0.f;
            if (j < end && j != i) {
                b = a.atoms[j];
                const float dx = b.x - p.x, dy = b.y - p.y, dz = b.z - p.z;
                const float lim = reach + b.w;
                const float d2 = dx * dx + dy * dy + dz * dz;
                keep = d2 < lim * lim;
                ratio = __fdividef(d2, lim * lim); // the band is a heuristic: fast math

            }
            const unsigned m = __ballot_sync(kFull, keep);
            if (keep) {
                const int k = n_list + __popc(m & lt_mask);
                const float e = __fadd_rn(a.probe, b.w);
                list[k] = make_float4(b.x, b.y, b.z, -__fmul_rn(e, e));
                band[k] = (unsigned char)min(kBuckets - 1,
                                             (int)(kBuckets * ratio * rsqrtf(fmaxf(ratio, 1e-20f))));
            }
            n_list += __popc(m);
            if (beg + 32 >= end) {
                ++row;
                pos = 0;
            } else {
                pos += 32;
            }
        }
        if (walk_done) {
            // the atom itself, last in the last list (it occludes its own
            // dots only through rounding at very large coordinates)
            if (lane == 0) {
                const float e = __fadd_rn(a.probe, p.w);
                list[n_list] = make_float4(p.x, p.y, p.z, -__fmul_rn(e, e));
                band[n_list] = kBuckets - 1;
            }
            ++n_list;
        }
        __syncwarp();
        const int n_pairs = sort_into_pairs(list, band, s_count[warp], n_list, lane);
        test_list(a, list, n_pairs, n_list, open, g0, ng, p, ext, lane, tests);
        n_list = 0;
        __syncwarp();
        if (walk_done)
            break;
    }
    unsigned exposed = 0;
    for (int g = lane; g < ng; g += 32)
        exposed += __popc(open[g]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        exposed += __shfl_xor_sync(kFull, exposed, o);
        tests += __shfl_xor_sync(kFull, tests, o);
    }
    if (lane == 0) {
        a.counts[a.orig_index[i]] = exposed;
        if (a.tests)
            atomicAdd(a.tests, tests);
    }
}

cudaError_t launch_sasa(const SasaArgs &a, cudaStream_t st)
{
    if (a.n_atoms == 0)
        return cudaSuccess;
    const int blocks = (a.n_atoms + kSasaWarps - 1) / kSasaWarps;
    sasa_kernel<<<blocks, kSasaWarps * 32, 0, st>>>(a);
    count_launch();
    return cudaGetLastError();
}

} // namespace rsx
