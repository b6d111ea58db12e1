// Debye algorithm handle behind the C ABI (include/rsx.h): host logic for
// calc / recalc / commit / revert / backward.  Replaces saxs_cl_gpu<float>
// (resaxslib/src/saxs_alg_cl_gpu_pt_wf.cpp) with a CUDA runtime layer: one
// stream per handle, device-resident bodies in type-sorted order, FP64
// running curve.
#include "rsx_autotune.h"
#include "rsx_host.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

using namespace rsx;

namespace {

unsigned type_of(const rsx_body &b)
{
    unsigned t;
    std::memcpy(&t, &b.w, sizeof t); // utils.hpp:61-66
    return t;
}

// Layout of the bodies on the device: type-sorted order, block tiles and
// the forward work items (upper triangle of block pairs, J runs of one type
// grouped `jchunk` at a time).
struct Layout {
    std::vector<unsigned> types;  // caller order
    std::vector<int> perm;        // sorted -> caller
    std::vector<int> inv;         // caller -> sorted
    std::vector<int> type_start;  // [T+1]
    std::vector<int> type_count;  // [T]
    std::vector<BlockDesc> blocks;
    std::vector<PairItem> items;     // forward
    std::vector<PairItem> adj_items; // adjoint (no q-slab grid dimension)
};

std::vector<PairItem> make_items(const std::vector<BlockDesc> &blocks, int jchunk)
{
    std::vector<PairItem> items;
    jchunk = std::max(jchunk, 1);
    const int nb = (int)blocks.size();
    for (int bi = 0; bi < nb; ++bi) {
        int bj = bi;
        while (bj < nb) {
            const int t = blocks[bj].type;
            int end = bj;
            while (end < nb && blocks[end].type == t && end - bj < jchunk)
                ++end;
            items.push_back(PairItem{bi, bj, end, 0});
            bj = end;
        }
    }
    return items;
}

// Item range [lo, hi) of shard `shard` of `n_shards`: contiguous runs of the
// forward items balanced by pair count (|I-block| x sum of |J-blocks|), so a
// shard's work differs from the mean by at most one item's.
std::pair<int, int> shard_items(const Layout &L, int shard, int n_shards)
{
    const int n = (int)L.items.size();
    std::vector<double> prefix(n + 1, 0.0);
    for (int i = 0; i < n; ++i) {
        const PairItem &it = L.items[i];
        double w = 0.0;
        for (int b = it.bj_begin; b < it.bj_end; ++b)
            w += (double)L.blocks[b].len;
        prefix[i + 1] = prefix[i] + w * L.blocks[it.bi].len;
    }
    auto bound = [&](int s) {
        if (s <= 0)
            return 0;
        if (s >= n_shards)
            return n;
        const double target = prefix[n] * s / n_shards;
        return (int)(std::lower_bound(prefix.begin(), prefix.end(), target) - prefix.begin());
    };
    const int lo = std::min(bound(shard), n), hi = std::min(bound(shard + 1), n);
    return {lo, std::max(lo, hi)};
}

void build_layout(Layout &L, const rsx_body *bodies, int n, int n_types, int max_items,
                  int min_adj_items)
{
    L.types.resize(n);
    for (int i = 0; i < n; ++i)
        L.types[i] = type_of(bodies[i]);
    L.type_count.assign(n_types, 0);
    for (int i = 0; i < n; ++i)
        L.type_count[L.types[i]]++;
    L.type_start.assign(n_types + 1, 0);
    for (int t = 0; t < n_types; ++t)
        L.type_start[t + 1] = L.type_start[t] + L.type_count[t];
    L.perm.resize(n);
    L.inv.resize(n);
    std::vector<int> fill(L.type_start.begin(), L.type_start.end() - 1);
    for (int i = 0; i < n; ++i) {
        const int s = fill[L.types[i]]++;
        L.perm[s] = i;
        L.inv[i] = s;
    }
    L.blocks.clear();
    for (int t = 0; t < n_types; ++t)
        for (int s = L.type_start[t]; s < L.type_start[t + 1]; s += kBlockAtoms)
            L.blocks.push_back(BlockDesc{s, std::min(kBlockAtoms, L.type_start[t + 1] - s), t, 0});
    // grow the J run per item until the item count fits; it cannot drop below
    // one item per (I-block, type run), reached once jchunk >= n_blocks
    const int nb = (int)L.blocks.size();
    int jchunk = 1;
    L.items = make_items(L.blocks, jchunk);
    while ((int)L.items.size() > max_items && jchunk < nb) {
        jchunk = std::min(jchunk * 2, nb);
        L.items = make_items(L.blocks, jchunk);
    }
    // adjoint: as few items as keep every SM busy (fewer FP64 gradient flushes)
    int aj = 1;
    L.adj_items = make_items(L.blocks, aj);
    for (;;) {
        if (aj * 2 > nb)
            break;
        auto next = make_items(L.blocks, aj * 2);
        if ((int)next.size() < min_adj_items)
            break;
        aj *= 2;
        L.adj_items.swap(next);
    }
}

bool detect_uniform(const std::vector<float> &q, float *dq_out)
{
    const int n = (int)q.size();
    if (n == 1) {
        *dq_out = 0.f;
        return true;
    }
    const double q0 = q[0];
    const double dq = ((double)q[n - 1] - q0) / (n - 1);
    for (int k = 0; k < n; ++k) {
        const double ideal = q0 + k * dq;
        if (std::fabs((double)q[k] - ideal) > 4e-7 * std::fabs((double)q[k]) + 1e-30)
            return false;
    }
    *dq_out = (float)dq;
    return true;
}

} // namespace

struct rsx_debye {
    int device = -1;
    cudaStream_t st = nullptr;
    cudaEvent_t ev_k0 = nullptr, ev_k1 = nullptr, ev_c0 = nullptr, ev_c1 = nullptr;
    AuxStream aux{nullptr, nullptr, nullptr}; // tail slab of the wide forward
    bool timing = false;
    int n = 0, n_q = 0, n_types = 0;
    std::vector<float> q, ff;
    bool ff_on_device = false; // d_ff holds ff
    bool uniform = false;
    float dq = 0.f;
    float lo[3] = {0.f, 0.f, 0.f}, hi[3] = {0.f, 0.f, 0.f}; // extent of the device bodies
    int q_slab = 32;
    int pairs_per_step = 2; // wide forward main slabs of 128 q and more: 2 or 4
    int max_items = 16384;
    bool autotune = false, tuned = false;
    bool pair_tables = true; // tabulated adjoint, gridded non-uniform forward

    // implicit water (caller order)
    float water_weight = 0.f;
    int water_index = 0;
    std::vector<float> rsasa;
    bool params_dirty = true;

    Layout L;
    bool have_layout = false;
    unsigned layout_version = 0;
    std::vector<rsx_body> cur;        // caller-order bodies of the current state
    bool computing = false;

    // checkpoint (commit / revert)
    bool have_saved = false;
    std::vector<rsx_body> saved_bodies;
    std::vector<float> saved_ff, saved_rsasa;
    float saved_ww = 0.f;
    int saved_wi = 0;
    unsigned saved_layout_version = 0;

    // device buffers
    float4 *d_pos = nullptr, *d_pos_saved = nullptr;
    float *d_rsasa = nullptr;
    float *d_ff = nullptr, *d_q = nullptr;
    BlockDesc *d_blocks = nullptr;
    PairItem *d_items = nullptr, *d_adj_items = nullptr;
    size_t items_cap = 0, adj_cap = 0;
    double *d_partial = nullptr;
    size_t partial_cap = 0; // doubles
    double *d_iq64 = nullptr, *d_iq64_saved = nullptr;
    float *d_iq32 = nullptr;
    int *d_type_count = nullptr;
    double *d_rsasa_sum = nullptr;
    size_t blocks_cap = 0;
    // incremental
    unsigned char *d_moved = nullptr; // packed moved_new | moved_idx | tiles
    size_t moved_cap = 0;
    // adjoint
    double *d_grad = nullptr;
    float *d_lambda = nullptr;
    float4 *d_adj_tab = nullptr; // tabulated pair functions (no water)
    size_t adj_tab_cap = 0;      // float4
    // gridded pair-distance histograms of the non-uniform forward
    double *d_grid = nullptr;
    size_t grid_cap = 0; // doubles

    // pinned staging
    float4 *h_pos = nullptr;
    float *h_iq = nullptr;
    double *h_iq64 = nullptr;
    double *h_grad = nullptr;
    unsigned char *h_moved = nullptr;
    float *h_rsasa = nullptr;

    // water sums (sorted by type)
    std::vector<double> rsasa_sum;
    double rsasa_sq = 0.0, rsasa_tot = 0.0;

    float last_ms_kernel = 0.f, last_ms_call = 0.f;
};

namespace {

template <class T>
rsx_status ensure(T **p, size_t &cap, size_t count, const char *what)
{
    if (*p && cap >= count)
        return RSX_OK;
    dev_free(*p);
    *p = nullptr;
    cap = 0;
    RSX_TRY(dev_alloc((void **)p, sizeof(T) * std::max<size_t>(count, 1), what));
    cap = count;
    return RSX_OK;
}

rsx_status check_bodies(const rsx_debye *h, const rsx_body *b, size_t count)
{
    for (size_t i = 0; i < count; ++i) {
        if (type_of(b[i]) >= (unsigned)h->n_types)
            return fail(RSX_INVALID_ARG, "body " + std::to_string(i) + " has factor index " +
                                             std::to_string(type_of(b[i])) + " >= n_factors " +
                                             std::to_string(h->n_types));
    }
    return RSX_OK;
}

void water_sums(rsx_debye *h)
{
    h->rsasa_sum.assign(h->n_types, 0.0);
    h->rsasa_sq = h->rsasa_tot = 0.0;
    for (int i = 0; i < h->n; ++i) {
        const double r = h->rsasa[i];
        h->rsasa_sum[h->L.types[i]] += r;
        h->rsasa_sq += r * r;
        h->rsasa_tot += r;
    }
}

bool has_water(const rsx_debye *h) { return h->water_weight != 0.f; }

// q slab of the general kernels (the adjoint, the delta and the non-wide
// forward): water keeps two accumulator sets in registers there.
int slab_for(const rsx_debye *h)
{
    int qs = std::min(h->q_slab, 128); // 192 selects the wider forward slabs only
    if (has_water(h) && qs > 16)
        qs = 16;
    if (!h->uniform && qs > 32)
        qs = 32; // the direct-sine path has no wide variant
    return qs;
}

// q slab of the forward: on uniform grids the wide slabs (q_slab 64 / 128)
// also carry the water term.
int forward_slab(const rsx_debye *h)
{
    return (h->uniform && h->q_slab >= 64) ? h->q_slab : slab_for(h);
}

// Re-derives the device layout when the body types changed.
// `same`: the bodies' types match the current layout (scan_bodies).
rsx_status update_layout(rsx_debye *h, const rsx_body *bodies, bool same)
{
    if (same && h->have_layout)
        return RSX_OK;
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device);
    build_layout(h->L, bodies, h->n, h->n_types, h->max_items, sms * 64);
    RSX_TRY(ensure(&h->d_blocks, h->blocks_cap, h->L.blocks.size(), "blocks"));
    RSX_TRY(ensure(&h->d_items, h->items_cap, h->L.items.size(), "items"));
    RSX_TRY(ensure(&h->d_adj_items, h->adj_cap, h->L.adj_items.size(), "adjoint items"));
    // (an incremental step grows it to its own need in delta_update)
    const size_t need = h->L.items.size() * (size_t)h->n_q;
    RSX_TRY(ensure(&h->d_partial, h->partial_cap, need, "partial sums"));
    RSX_TRY_CUDA(cudaMemcpyAsync(h->d_blocks, h->L.blocks.data(),
                                 sizeof(BlockDesc) * h->L.blocks.size(), cudaMemcpyHostToDevice,
                                 h->st),
                 "upload blocks");
    RSX_TRY_CUDA(cudaMemcpyAsync(h->d_items, h->L.items.data(),
                                 sizeof(PairItem) * h->L.items.size(), cudaMemcpyHostToDevice,
                                 h->st),
                 "upload items");
    RSX_TRY_CUDA(cudaMemcpyAsync(h->d_adj_items, h->L.adj_items.data(),
                                 sizeof(PairItem) * h->L.adj_items.size(),
                                 cudaMemcpyHostToDevice, h->st),
                 "upload adjoint items");
    RSX_TRY_CUDA(cudaMemcpyAsync(h->d_type_count, h->L.type_count.data(),
                                 sizeof(int) * h->n_types, cudaMemcpyHostToDevice, h->st),
                 "upload type counts");
    // pageable host vectors above: make them safe to reuse
    RSX_TRY_CUDA(cudaStreamSynchronize(h->st), "layout upload");
    h->have_layout = true;
    h->layout_version++;
    return RSX_OK;
}

rsx_status upload_water(rsx_debye *h)
{
    if (!has_water(h))
        return RSX_OK;
    water_sums(h);
    for (int s = 0; s < h->n; ++s)
        h->h_rsasa[s] = h->rsasa[h->L.perm[s]];
    RSX_TRY_CUDA(cudaMemcpyAsync(h->d_rsasa, h->h_rsasa, sizeof(float) * h->n,
                                 cudaMemcpyHostToDevice, h->st),
                 "upload rsasa");
    RSX_TRY_CUDA(cudaMemcpyAsync(h->d_rsasa_sum, h->rsasa_sum.data(), sizeof(double) * h->n_types,
                                 cudaMemcpyHostToDevice, h->st),
                 "upload rsasa sums");
    return RSX_OK;
}

// One pass over a full set of caller bodies: factor indices (an error names
// the first bad one), whether the types match the device layout, and the
// bounding box.  The box is the extent of the device bodies: reset by a full
// upload, grown by moves (never shrunk until the next full upload, so it stays
// an upper bound).
rsx_status scan_bodies(rsx_debye *h, const rsx_body *b, bool *same_types)
{
    bool same = h->have_layout && (int)h->L.types.size() == h->n;
    float lo[3] = {3.4e38f, 3.4e38f, 3.4e38f}, hi[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
    for (int i = 0; i < h->n; ++i) {
        const unsigned t = type_of(b[i]);
        if (t >= (unsigned)h->n_types)
            return fail(RSX_INVALID_ARG, "body " + std::to_string(i) + " has factor index " +
                                             std::to_string(t) + " >= n_factors " +
                                             std::to_string(h->n_types));
        same = same && t == h->L.types[i];
        lo[0] = std::min(lo[0], b[i].x);
        hi[0] = std::max(hi[0], b[i].x);
        lo[1] = std::min(lo[1], b[i].y);
        hi[1] = std::max(hi[1], b[i].y);
        lo[2] = std::min(lo[2], b[i].z);
        hi[2] = std::max(hi[2], b[i].z);
    }
    for (int d = 0; d < 3; ++d) {
        h->lo[d] = lo[d];
        h->hi[d] = hi[d];
    }
    *same_types = same;
    return RSX_OK;
}

void grow_extent(rsx_debye *h, const rsx_body *b, unsigned n)
{
    for (unsigned i = 0; i < n; ++i) {
        const float x[3] = {b[i].x, b[i].y, b[i].z};
        for (int d = 0; d < 3; ++d) {
            h->lo[d] = std::min(h->lo[d], x[d]);
            h->hi[d] = std::max(h->hi[d], x[d]);
        }
    }
}

// theta_level() of the tracked bounding box (the seeds may skip the range
// reduction where it allows; the result is the same bit for bit).
int small_theta(const rsx_debye *h)
{
    if (!h->uniform || h->n < 2)
        return 0;
    double d2 = 0.0;
    for (int d = 0; d < 3; ++d) {
        const double e = (double)h->hi[d] - (double)h->lo[d];
        if (!(e >= 0.0) || !std::isfinite(e))
            return 0;
        d2 += e * e;
    }
    return theta_level(true, (double)h->dq, std::sqrt(d2));
}

// A uniform grid that starts at q = 0 with q[1] == dq: the wide launches
// skip that q (past_q0), and their first seeds take sin/cos(q[1] r) from the
// step's sin/cos(dq r).
bool q0_free(const rsx_debye *h)
{
    return h->uniform && h->n_q > 1 && h->q[0] == 0.f && h->q[1] == h->dq;
}

DebyeArgs debye_args(rsx_debye *h)
{
    DebyeArgs a{};
    a.pos = h->d_pos;
    a.rsasa = has_water(h) ? h->d_rsasa : nullptr;
    a.ff = h->d_ff;
    a.q = h->d_q;
    a.blocks = h->d_blocks;
    a.items = h->d_items;
    a.partial = h->d_partial;
    a.n = h->n;
    a.n_q = h->n_q;
    a.n_types = h->n_types;
    a.n_items = (int)h->L.items.size();
    a.dq = h->dq;
    a.small_theta = small_theta(h);
    a.q0_free = q0_free(h) ? 1 : 0;
    a.pairs4 = h->pairs_per_step == 4 ? 1 : 0;
    a.water_weight = h->water_weight;
    a.water_index = h->water_index;
    return a;
}

AssembleArgs assemble_args(rsx_debye *h, int n_parts, int accumulate)
{
    AssembleArgs a{};
    a.partial = h->d_partial;
    a.ff = h->d_ff;
    a.q = h->d_q;
    a.type_count = h->d_type_count;
    a.rsasa_sum = h->d_rsasa_sum;
    a.rsasa_sq_sum = h->rsasa_sq;
    a.rsasa_total = h->rsasa_tot;
    a.n_q = h->n_q;
    a.n_types = h->n_types;
    a.n_parts = n_parts;
    a.water_weight = h->water_weight;
    a.water_index = h->water_index;
    a.has_water = has_water(h) ? 1 : 0;
    a.iq64 = h->d_iq64;
    a.iq32 = h->d_iq32;
    a.accumulate = accumulate;
    return a;
}

// Forward over the device-resident bodies (no host transfers).
// Node grid of the gridded forward / tabulated adjoint: nodes r = b h covering
// the tracked bounding-box diagonal with q_max h <= 0.05.  False for an empty
// or non-finite extent.
bool pair_grid(const rsx_debye *h, double *nodes, double *step)
{
    double d2 = 0.0;
    for (int d = 0; d < 3; ++d) {
        const double e = (double)h->hi[d] - (double)h->lo[d];
        if (!std::isfinite(e))
            return false;
        d2 += e > 0.0 ? e * e : 0.0;
    }
    double q_max = 0.0;
    for (float q : h->q)
        q_max = std::max(q_max, std::fabs((double)q));
    const double r_max = std::sqrt(d2) * 1.0001 + 1e-3;
    *nodes = std::max(16.0, std::ceil(r_max * q_max / 0.05) + 2.0);
    *step = r_max / (*nodes - 2.0);
    return *step > 0.0 && std::isfinite(*step);
}

unsigned present_types(const rsx_debye *h)
{
    unsigned mask = 0;
    for (int t = 0; t < h->n_types && t < 32; ++t)
        if (h->L.type_count[t] > 0)
            mask |= 1u << t;
    return mask;
}

rsx_status forward_device(rsx_debye *h)
{
    DebyeArgs a = debye_args(h);
    // non-uniform grids: the gridded pair-distance distribution
    const bool water = has_water(h);
    double nodes = 0.0, step = 0.0;
    const bool gridded = h->pair_tables && !h->uniform && h->n_types <= 32 &&
                         pair_grid(h, &nodes, &step) && nodes <= forward_grid_max_nodes(water);
    if (gridded)
        RSX_TRY(ensure(&h->d_grid, h->grid_cap,
                       forward_grid_doubles(h->n_types, h->n_q, (int)nodes, water),
                       "forward histograms"));
    if (h->timing)
        RSX_TRY_CUDA(cudaEventRecord(h->ev_k0, h->st), "event");
    if (gridded)
        RSX_LAUNCH(launch_forward_grid(a, h->d_grid, (int)nodes, (float)step, present_types(h),
                                       water, h->st),
                   "forward kernels");
    else
        RSX_LAUNCH(launch_forward(a, forward_slab(h), h->uniform, has_water(h), h->st, &h->aux),
                   "forward kernel");
    if (h->timing)
        RSX_TRY_CUDA(cudaEventRecord(h->ev_k1, h->st), "event");
    RSX_LAUNCH(launch_assemble(assemble_args(h, gridded ? 1 : a.n_items, 0), h->st),
               "assemble kernel");
    return RSX_OK;
}

rsx_status finish_timing(rsx_debye *h)
{
    if (!h->timing)
        return RSX_OK;
    RSX_TRY_CUDA(cudaEventRecord(h->ev_c1, h->st), "event");
    RSX_TRY_CUDA(cudaEventSynchronize(h->ev_c1), "event sync");
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, h->ev_k0, h->ev_k1) == cudaSuccess)
        h->last_ms_kernel = ms;
    if (cudaEventElapsedTime(&ms, h->ev_c0, h->ev_c1) == cudaSuccess)
        h->last_ms_call = ms;
    return RSX_OK;
}

rsx_status read_curve(rsx_debye *h, float *out_iq)
{
    RSX_TRY_CUDA(cudaMemcpyAsync(h->h_iq, h->d_iq32, sizeof(float) * h->n_q,
                                 cudaMemcpyDeviceToHost, h->st),
                 "read curve");
    RSX_TRY(finish_timing(h));
    RSX_TRY_CUDA(cudaStreamSynchronize(h->st), "calc");
    if (out_iq)
        std::memcpy(out_iq, h->h_iq, sizeof(float) * h->n_q);
    return RSX_OK;
}

// Picks the tile shape of the forward for this problem class -- the q-slab
// plan and, for the wide slabs of 128 q and more, the pairs a thread steps
// together -- as the cached winner, or the fastest candidate timed here (two
// timed runs each, after a warm-up) on the bodies just uploaded.  The cache
// holds q_slab + 1000 * (pairs_per_step == 4).
rsx_status tune_slab(rsx_debye *h)
{
    h->tuned = true;
    const std::string key = autotune_key(h->device, "forward", h->n, h->n_q, h->n_types,
                                         h->uniform, has_water(h));
    int qs = 0;
    if (autotune_lookup(key, &qs)) {
        h->q_slab = qs % 1000;
        h->pairs_per_step = qs >= 1000 ? 4 : 2;
        return RSX_OK;
    }
    std::vector<int> cands = {16, 32};
    if (h->uniform) {
        cands.push_back(64);
        cands.push_back(128);
        if (!has_water(h)) {
            cands.push_back(1128);
            if (h->n_q >= 192) {
                cands.push_back(192);
                cands.push_back(1192);
            }
        }
    }
    cudaEvent_t e0, e1;
    RSX_TRY_CUDA(cudaEventCreate(&e0), "event");
    RSX_TRY_CUDA(cudaEventCreate(&e1), "event");
    float best = 1e30f;
    int best_qs = h->q_slab;
    rsx_status st = RSX_OK;
    const bool timing = h->timing;
    h->timing = false;
    for (int c : cands) {
        h->q_slab = c % 1000;
        h->pairs_per_step = c >= 1000 ? 4 : 2;
        float t_min = 1e30f;
        for (int rep = 0; rep < 3 && st == RSX_OK; ++rep) {
            cudaEventRecord(e0, h->st);
            st = forward_device(h);
            cudaEventRecord(e1, h->st);
            if (cudaEventSynchronize(e1) != cudaSuccess)
                st = fail(RSX_CUDA_ERROR, "autotune run failed");
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (rep > 0)
                t_min = std::min(t_min, ms);
        }
        if (st != RSX_OK)
            break;
        if (t_min < best) {
            best = t_min;
            best_qs = c;
        }
    }
    h->timing = timing;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    h->q_slab = best_qs % 1000;
    h->pairs_per_step = best_qs >= 1000 ? 4 : 2;
    if (st == RSX_OK)
        autotune_store(key, best_qs);
    return st;
}

// Full calculation from caller-order bodies.
rsx_status upload_all(rsx_debye *h, const rsx_body *bodies)
{
    bool same = false;
    RSX_TRY(scan_bodies(h, bodies, &same));
    RSX_TRY(update_layout(h, bodies, same));
    for (int s = 0; s < h->n; ++s) {
        const rsx_body &b = bodies[h->L.perm[s]];
        h->h_pos[s] = make_float4(b.x, b.y, b.z, b.w);
    }
    RSX_TRY_CUDA(cudaMemcpyAsync(h->d_pos, h->h_pos, sizeof(float4) * h->n,
                                 cudaMemcpyHostToDevice, h->st),
                 "upload bodies");
    if (!h->ff_on_device) {
        RSX_TRY_CUDA(cudaMemcpyAsync(h->d_ff, h->ff.data(), sizeof(float) * h->ff.size(),
                                     cudaMemcpyHostToDevice, h->st),
                     "upload factors");
        h->ff_on_device = true;
    }
    RSX_TRY(upload_water(h));
    return RSX_OK;
}

rsx_status full_calc(rsx_debye *h, const rsx_body *bodies)
{
    RSX_TRY(upload_all(h, bodies));
    if (h->autotune && !h->tuned)
        RSX_TRY(tune_slab(h));
    RSX_TRY(forward_device(h));
    h->cur.assign(bodies, bodies + h->n);
    h->params_dirty = false;
    h->computing = true;
    return RSX_OK;
}

rsx_status begin_call(rsx_debye *h, bool mark_call = true)
{
    if (!h)
        return fail(RSX_ALG_NOT_INITIALIZED, "null rsx_debye handle");
    RSX_TRY_CUDA(cudaSetDevice(h->device), "cudaSetDevice");
    if (h->timing && mark_call)
        RSX_TRY_CUDA(cudaEventRecord(h->ev_c0, h->st), "event");
    return RSX_OK;
}

// Incremental update for moved caller indices `idx` with new bodies `moved`.
rsx_status delta_update(rsx_debye *h, const rsx_body *moved, const unsigned *idx, unsigned k)
{
    // moved list grouped by type (counting sort), tiles of <= 128 per type
    std::vector<int> cnt(h->n_types + 1, 0);
    for (unsigned m = 0; m < k; ++m)
        cnt[type_of(moved[m]) + 1]++;
    for (int t = 0; t < h->n_types; ++t)
        cnt[t + 1] += cnt[t];
    std::vector<int> order(k);
    {
        std::vector<int> fill(cnt.begin(), cnt.end() - 1);
        for (unsigned m = 0; m < k; ++m)
            order[fill[type_of(moved[m])]++] = (int)m;
    }
    // Each type's run is cut into near-equal tiles, longest first: at most
    // kDeltaTile bodies for the wide kernel (its chain states between the two
    // slabs are kept per tile body; the tiles are split over up to
    // kDeltaGroups CTA groups), else at most max(8, k / 8).
    std::vector<BlockDesc> tiles;
    const bool wide = h->uniform && slab_for(h) >= 64;
    const int cap = wide ? kDeltaTile : std::min(kBlockAtoms, std::max(8, (int)((k + 7) / 8)));
    for (int t = 0; t < h->n_types; ++t) {
        const int c = cnt[t + 1] - cnt[t];
        if (c == 0)
            continue;
        const int nt = (c + cap - 1) / cap, base = c / nt, extra = c % nt;
        for (int j = 0, s = cnt[t]; j < nt; ++j) {
            const int len = base + (j < extra ? 1 : 0);
            tiles.push_back(BlockDesc{s, len, t, 0});
            s += len;
        }
    }
    std::stable_sort(tiles.begin(), tiles.end(),
                     [](const BlockDesc &x, const BlockDesc &y) { return x.len > y.len; });
    const size_t off_idx = sizeof(float4) * k;
    const size_t off_tiles = (off_idx + sizeof(int) * k + 15) & ~size_t(15);
    const size_t bytes = off_tiles + sizeof(BlockDesc) * tiles.size();
    if (bytes > h->moved_cap) {
        dev_free(h->d_moved);
        host_free_pinned(h->h_moved);
        h->d_moved = nullptr;
        h->h_moved = nullptr;
        h->moved_cap = 0;
        const size_t cap = std::max<size_t>(bytes * 2, 64 * 1024);
        RSX_TRY(dev_alloc((void **)&h->d_moved, cap, "moved list"));
        RSX_TRY(host_alloc_pinned((void **)&h->h_moved, cap, "moved staging"));
        h->moved_cap = cap;
    }
    // the pinned staging buffer may still feed the previous step's copy
    RSX_TRY_CUDA(cudaStreamSynchronize(h->st), "recalc staging");
    float4 *mv = reinterpret_cast<float4 *>(h->h_moved);
    int *mi = reinterpret_cast<int *>(h->h_moved + off_idx);
    for (unsigned s = 0; s < k; ++s) {
        const rsx_body &b = moved[order[s]];
        mv[s] = make_float4(b.x, b.y, b.z, b.w);
        mi[s] = h->L.inv[idx[order[s]]];
    }
    std::memcpy(h->h_moved + off_tiles, tiles.data(), sizeof(BlockDesc) * tiles.size());
    RSX_TRY_CUDA(cudaMemcpyAsync(h->d_moved, h->h_moved, bytes, cudaMemcpyHostToDevice, h->st),
                 "upload moved list");
    DeltaArgs a{};
    a.pos_old = h->d_pos;
    a.moved_new = reinterpret_cast<const float4 *>(h->d_moved);
    a.moved_idx = reinterpret_cast<const int *>(h->d_moved + off_idx);
    a.blocks = h->d_blocks;
    a.mtiles = reinterpret_cast<const BlockDesc *>(h->d_moved + off_tiles);
    a.ff = h->d_ff;
    a.q = h->d_q;
    a.n = h->n;
    a.k = (int)k;
    a.n_q = h->n_q;
    a.n_types = h->n_types;
    a.n_blocks = (int)h->L.blocks.size();
    a.n_mtiles = (int)tiles.size();
    a.max_groups = kDeltaGroups;
    a.dq = h->dq;
    a.q0_free = q0_free(h) ? 1 : 0;
    // one partial row per static block and moved-list group
    RSX_TRY(ensure(&h->d_partial, h->partial_cap,
                   (size_t)delta_parts(a, slab_for(h), h->uniform) * h->n_q, "partial sums"));
    a.partial = h->d_partial;
    // the extent already holds the moved bodies' new positions (recalc_common
    // grows it first), so the level covers the pairs before and after the move
    a.small_theta = small_theta(h);
    int *d_idx = reinterpret_cast<int *>(h->d_moved + off_idx);
    if (h->timing)
        RSX_TRY_CUDA(cudaEventRecord(h->ev_k0, h->st), "event");
    RSX_LAUNCH(launch_delta(a, slab_for(h), h->uniform, h->st, &h->aux), "delta kernel");
    if (h->timing)
        RSX_TRY_CUDA(cudaEventRecord(h->ev_k1, h->st), "event");
    AssembleArgs as = assemble_args(h, delta_parts(a, slab_for(h), h->uniform), 1);
    as.apply_pos = h->d_pos;
    as.apply_new = a.moved_new;
    as.apply_idx = d_idx;
    as.apply_k = (int)k;
    RSX_LAUNCH(launch_assemble(as, h->st), "assemble delta and apply moves");
    return RSX_OK;
}

rsx_status recalc_common(rsx_debye *h, const rsx_body *moved, const unsigned *idx, unsigned k,
                         float *out_iq)
{
    if (!h->computing)
        return fail(RSX_NO_INITIAL_CALC,
                    "recalc called before an initial call to calc (saxs_alg_cl_gpu_pt_wf.cpp:471)");
    RSX_TRY(check_bodies(h, moved, k));
    for (unsigned m = 0; m < k; ++m) {
        if (idx[m] >= (unsigned)h->n)
            return fail(RSX_INVALID_ARG, "moved index out of range");
        if (type_of(moved[m]) != h->L.types[idx[m]])
            return fail(RSX_INVALID_ARG, "recalc cannot change the type of a body");
    }
    {
        std::vector<unsigned> s(idx, idx + k);
        std::sort(s.begin(), s.end());
        if (std::adjacent_find(s.begin(), s.end()) != s.end())
            return fail(RSX_INVALID_ARG, "moved indices must be distinct");
    }
    if (h->params_dirty || has_water(h) || (size_t)k * 3 > (size_t)h->n) {
        // dirty params (saxs_alg_cl_gpu_pt_wf.cpp:479-504), water factors, or
        // most bodies moved: a full recompute is as cheap and exact
        std::vector<rsx_body> next = h->cur;
        for (unsigned m = 0; m < k; ++m)
            next[idx[m]] = moved[m];
        RSX_TRY(full_calc(h, next.data()));
    } else if (k > 0) {
        grow_extent(h, moved, k); // an upper bound of every pair distance, old and new
        RSX_TRY(delta_update(h, moved, idx, k));
        for (unsigned m = 0; m < k; ++m)
            h->cur[idx[m]] = moved[m];
    }
    return read_curve(h, out_iq);
}

rsx_status release(rsx_debye *h)
{
    if (!h)
        return RSX_OK;
    DeviceGuard g(h->device);
    if (h->st)
        cudaStreamSynchronize(h->st);
    if (h->aux.stream)
        cudaStreamSynchronize(h->aux.stream);
    void *dev[] = {h->d_pos,        h->d_pos_saved, h->d_rsasa,      h->d_ff,
                   h->d_q,          h->d_blocks,    h->d_items,      h->d_adj_items,
                   h->d_partial,    h->d_iq64,      h->d_iq64_saved, h->d_iq32,
                   h->d_type_count, h->d_rsasa_sum, h->d_moved,      h->d_grad,
                   h->d_lambda,     h->d_adj_tab,   h->d_grid};
    for (void *p : dev)
        dev_free(p);
    void *pinned[] = {h->h_pos, h->h_iq, h->h_iq64, h->h_grad, h->h_moved, h->h_rsasa};
    for (void *p : pinned)
        host_free_pinned(p);
    cudaEvent_t evs[] = {h->ev_k0, h->ev_k1, h->ev_c0, h->ev_c1, h->aux.fork, h->aux.join};
    for (auto e : evs)
        if (e)
            cudaEventDestroy(e);
    if (h->aux.stream)
        cudaStreamDestroy(h->aux.stream);
    if (h->st)
        cudaStreamDestroy(h->st);
    delete h;
    return RSX_OK;
}

} // namespace

extern "C" {

void rsx_debye_default_options(rsx_debye_options *o)
{
    if (!o)
        return;
    std::memset(o, 0, sizeof *o);
    o->device = -1;
}

rsx_status rsx_debye_create(const float *q, int n_q, const float *t_factors, int n_factors,
                            int n_bodies, const rsx_debye_options *opts, rsx_debye **out)
{
    if (!out)
        return fail(RSX_INVALID_ARG, "out handle pointer is null");
    *out = nullptr;
    if (!q || !t_factors || n_q <= 0 || n_factors <= 0 || n_bodies < 0)
        return fail(RSX_INVALID_ARG, "q, factor table and sizes must be non-null / positive");
    if (n_factors > kMaxTypes)
        return fail(RSX_NOT_SUPPORTED, "at most " + std::to_string(kMaxTypes) + " factor types");
    rsx_debye_options o;
    rsx_debye_default_options(&o);
    if (opts)
        o = *opts;
    if (o.q_slab != 0 && o.q_slab != 8 && o.q_slab != 16 && o.q_slab != 32 && o.q_slab != 64 &&
        o.q_slab != 128 && o.q_slab != 192)
        return fail(RSX_INVALID_ARG, "q_slab must be 0, 8, 16, 32, 64, 128 or 192");
    if (o.pairs_per_step != 0 && o.pairs_per_step != 2 && o.pairs_per_step != 4)
        return fail(RSX_INVALID_ARG, "pairs_per_step must be 0, 2 or 4");
    int dev = -1;
    RSX_TRY(select_device(o.device, &dev));
    DeviceGuard g(dev);
    cudaSetDevice(dev);
    rsx_debye *h = new rsx_debye();
    h->device = dev;
    h->n = n_bodies;
    h->n_q = n_q;
    h->n_types = n_factors;
    h->q.assign(q, q + n_q);
    h->ff.assign(t_factors, t_factors + (size_t)n_q * n_factors);
    h->uniform = !o.force_general_q && detect_uniform(h->q, &h->dq);
    // default tile: the wide slabs (64 to 192 q per seed, by the plan's
    // measured costs) on uniform grids of 64 q or more, otherwise 32 / 16 / 8
    h->q_slab = o.q_slab ? o.q_slab
                         : (h->uniform && n_q >= 64 ? 192 : (n_q >= 32 ? 32 : (n_q >= 16 ? 16 : 8)));
    h->pairs_per_step = o.pairs_per_step ? o.pairs_per_step : 2;
    h->autotune = o.autotune != 0 && o.q_slab == 0 && o.pairs_per_step == 0;
    h->max_items = o.max_items > 0 ? o.max_items : 16384;
    h->timing = o.timing != 0;
    h->pair_tables = o.no_pair_tables == 0;
    h->rsasa.assign(n_bodies, 0.f);
    auto bail = [&](rsx_status s) {
        release(h);
        return s;
    };
    cudaError_t e = cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking);
    if (e != cudaSuccess)
        return bail(cuda_status(e, "cudaStreamCreate"));
    for (cudaEvent_t *ev : {&h->ev_k0, &h->ev_k1, &h->ev_c0, &h->ev_c1}) {
        e = cudaEventCreate(ev);
        if (e != cudaSuccess)
            return bail(cuda_status(e, "cudaEventCreate"));
    }
    e = cudaStreamCreateWithFlags(&h->aux.stream, cudaStreamNonBlocking);
    if (e != cudaSuccess)
        return bail(cuda_status(e, "cudaStreamCreate"));
    for (cudaEvent_t *ev : {&h->aux.fork, &h->aux.join}) {
        e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
        if (e != cudaSuccess)
            return bail(cuda_status(e, "cudaEventCreate"));
    }
    const size_t n = std::max(n_bodies, 1);
    rsx_status s;
#define RSX_ALLOC(ptr, bytes, what)                                                        \
    if ((s = dev_alloc((void **)&(ptr), (bytes), what)) != RSX_OK)                         \
        return bail(s);
#define RSX_PIN(ptr, bytes, what)                                                          \
    if ((s = host_alloc_pinned((void **)&(ptr), (bytes), what)) != RSX_OK)                 \
        return bail(s);
    RSX_ALLOC(h->d_pos, sizeof(float4) * n, "positions");
    RSX_ALLOC(h->d_pos_saved, sizeof(float4) * n, "saved positions");
    RSX_ALLOC(h->d_rsasa, sizeof(float) * n, "rsasa");
    RSX_ALLOC(h->d_ff, sizeof(float) * h->ff.size(), "factor table");
    RSX_ALLOC(h->d_q, sizeof(float) * n_q, "q");
    RSX_ALLOC(h->d_iq64, sizeof(double) * n_q, "curve");
    RSX_ALLOC(h->d_iq64_saved, sizeof(double) * n_q, "saved curve");
    RSX_ALLOC(h->d_iq32, sizeof(float) * n_q, "curve f32");
    RSX_ALLOC(h->d_type_count, sizeof(int) * n_factors, "type counts");
    RSX_ALLOC(h->d_rsasa_sum, sizeof(double) * n_factors, "rsasa sums");
    RSX_ALLOC(h->d_grad, sizeof(double) * 3 * n, "gradient");
    RSX_ALLOC(h->d_lambda, sizeof(float) * n_q, "lambda");
    RSX_PIN(h->h_pos, sizeof(float4) * n, "pinned bodies");
    RSX_PIN(h->h_iq, sizeof(float) * n_q, "pinned curve");
    RSX_PIN(h->h_iq64, sizeof(double) * n_q, "pinned curve f64");
    RSX_PIN(h->h_grad, sizeof(double) * 3 * n, "pinned gradient");
    RSX_PIN(h->h_rsasa, sizeof(float) * n, "pinned rsasa");
#undef RSX_ALLOC
#undef RSX_PIN
    e = cudaMemcpyAsync(h->d_q, h->q.data(), sizeof(float) * n_q, cudaMemcpyHostToDevice, h->st);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(h->d_iq64, 0, sizeof(double) * n_q, h->st);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(h->st);
    if (e != cudaSuccess)
        return bail(cuda_status(e, "handle initialisation"));
    *out = h;
    return ok();
}

rsx_status rsx_debye_destroy(rsx_debye *h)
{
    release(h);
    return ok();
}

rsx_status rsx_debye_set_factors(rsx_debye *h, const float *t_factors, int n_factors)
{
    if (!h)
        return fail(RSX_ALG_NOT_INITIALIZED, "null rsx_debye handle");
    if (!t_factors || n_factors != h->n_types)
        return fail(RSX_INVALID_ARG, "factor table must have the handle's n_factors columns");
    h->ff.assign(t_factors, t_factors + (size_t)h->n_q * n_factors);
    h->ff_on_device = false;
    h->params_dirty = true;
    return ok();
}

rsx_status rsx_debye_set_water(rsx_debye *h, float weight, int water_index, const float *rsasa)
{
    if (!h)
        return fail(RSX_ALG_NOT_INITIALIZED, "null rsx_debye handle");
    if (water_index < 0 || water_index >= h->n_types)
        return fail(RSX_INVALID_ARG, "water_index outside the factor table");
    if (!std::isfinite(weight))
        return fail(RSX_INVALID_ARG, "water weight must be finite");
    h->water_weight = weight;
    h->water_index = water_index;
    if (rsasa)
        h->rsasa.assign(rsasa, rsasa + h->n);
    h->params_dirty = true;
    return ok();
}

rsx_status rsx_debye_calc(rsx_debye *h, const rsx_body *bodies, float *out_iq)
{
    RSX_TRY(begin_call(h));
    if (!bodies && h->n > 0)
        return fail(RSX_INVALID_ARG, "bodies is null");
    RSX_TRY(full_calc(h, bodies)); // validates the bodies before any device work
    RSX_TRY(read_curve(h, out_iq));
    return ok();
}

rsx_status rsx_debye_calc_shard(rsx_debye *h, const rsx_body *bodies, int shard, int n_shards,
                                double *out_iq)
{
    RSX_TRY(begin_call(h));
    if (!bodies && h->n > 0)
        return fail(RSX_INVALID_ARG, "bodies is null");
    if (!out_iq || n_shards < 1 || shard < 0 || shard >= n_shards)
        return fail(RSX_INVALID_ARG, "need out_iq and 0 <= shard < n_shards");
    RSX_TRY(upload_all(h, bodies)); // validates the bodies before any device work
    // the device positions no longer hold a computed state: an incremental
    // call needs a full calc first
    h->computing = false;
    const auto range = shard_items(h->L, shard, n_shards);
    DebyeArgs a = debye_args(h);
    a.items = h->d_items + range.first;
    a.n_items = range.second - range.first;
    if (a.n_items > 0)
        RSX_LAUNCH(launch_forward(a, forward_slab(h), h->uniform, has_water(h), h->st),
                   "forward kernel");
    if (shard == 0) {
        RSX_LAUNCH(launch_assemble(assemble_args(h, a.n_items, 0), h->st), "assemble kernel");
    } else {
        RSX_TRY_CUDA(cudaMemsetAsync(h->d_iq64, 0, sizeof(double) * h->n_q, h->st), "clear");
        RSX_LAUNCH(launch_assemble(assemble_args(h, a.n_items, 1), h->st), "assemble kernel");
    }
    RSX_TRY_CUDA(cudaMemcpyAsync(h->h_iq64, h->d_iq64, sizeof(double) * h->n_q,
                                 cudaMemcpyDeviceToHost, h->st),
                 "read shard");
    RSX_TRY_CUDA(cudaStreamSynchronize(h->st), "calc shard");
    std::memcpy(out_iq, h->h_iq64, sizeof(double) * h->n_q);
    return ok();
}

int rsx_debug_theta_level(int uniform, double dq, double diag)
{
    return theta_level(uniform != 0, dq, diag);
}

rsx_status rsx_debug_chain_plan(int n_q, int *out)
{
    if (n_q <= 0 || !out)
        return fail(RSX_INVALID_ARG, "need n_q > 0 and an output");
    const ChainPlan p = chain_plan(n_q);
    out[0] = p.full;
    out[1] = p.rest_k0;
    out[2] = p.rest_main;
    out[3] = p.rest_tail;
    out[4] = p.rest ? 1 : 0;
    return ok();
}

rsx_status rsx_debug_wide_plan(int n_q, int q_slab, int *out)
{
    if (n_q <= 0 || !out || (q_slab != 64 && q_slab != 128 && q_slab != 192))
        return fail(RSX_INVALID_ARG, "need n_q > 0, q_slab 64, 128 or 192 and an output");
    const WidePlan p = wide_plan(n_q, q_slab);
    out[0] = p.main;
    out[1] = p.full;
    out[2] = p.tail_k0;
    out[3] = p.tail_len;
    out[4] = p.tail_w;
    return ok();
}

rsx_status rsx_debug_shard_items(const rsx_body *bodies, int n_bodies, int n_factors,
                                 int max_items, int n_shards, int *bounds, double *pairs)
{
    if ((!bodies && n_bodies > 0) || n_bodies < 0 || n_factors <= 0 || n_factors > kMaxTypes ||
        max_items <= 0 || n_shards < 1 || !bounds)
        return fail(RSX_INVALID_ARG, "bad shard arguments");
    for (int i = 0; i < n_bodies; ++i)
        if (type_of(bodies[i]) >= (unsigned)n_factors)
            return fail(RSX_INVALID_ARG, "type out of range");
    Layout L;
    build_layout(L, bodies, n_bodies, n_factors, max_items, 1);
    for (int sh = 0; sh < n_shards; ++sh) {
        const auto r = shard_items(L, sh, n_shards);
        bounds[sh] = r.first;
        bounds[sh + 1] = r.second;
        if (pairs) {
            // unordered pairs of distinct bodies in the shard's items
            double c = 0.0;
            for (int i = r.first; i < r.second; ++i) {
                const PairItem &it = L.items[i];
                const double li = L.blocks[it.bi].len;
                for (int b = it.bj_begin; b < it.bj_end; ++b)
                    c += (b == it.bi) ? li * (li - 1) / 2 : li * L.blocks[b].len;
            }
            pairs[sh] = c;
        }
    }
    return ok();
}

rsx_status rsx_debye_recalc_range(rsx_debye *h, const rsx_body *bodies, unsigned upd_start,
                                  unsigned upd_length, float *out_iq)
{
    RSX_TRY(begin_call(h));
    if ((size_t)upd_start + upd_length > (size_t)h->n)
        return fail(RSX_INVALID_ARG,
                    "update region exceeds the number of bodies (saxs_alg_cl_gpu_pt_wf.cpp:473)");
    if (!bodies && upd_length > 0)
        return fail(RSX_INVALID_ARG, "bodies is null");
    std::vector<unsigned> idx(upd_length);
    for (unsigned m = 0; m < upd_length; ++m)
        idx[m] = upd_start + m;
    RSX_TRY(recalc_common(h, bodies + upd_start, idx.data(), upd_length, out_iq));
    return ok();
}

rsx_status rsx_debye_recalc_indices(rsx_debye *h, const rsx_body *moved, const unsigned *idx,
                                    unsigned k, float *out_iq)
{
    RSX_TRY(begin_call(h));
    if (k > 0 && (!moved || !idx))
        return fail(RSX_INVALID_ARG, "moved bodies / indices are null");
    RSX_TRY(recalc_common(h, moved, idx, k, out_iq));
    return ok();
}

rsx_status rsx_debye_commit(rsx_debye *h)
{
    RSX_TRY(begin_call(h));
    if (!h->computing)
        return fail(RSX_NO_INITIAL_CALC, "commit called before an initial call to calc");
    RSX_TRY_CUDA(cudaMemcpyAsync(h->d_pos_saved, h->d_pos, sizeof(float4) * h->n,
                                 cudaMemcpyDeviceToDevice, h->st),
                 "save positions");
    RSX_TRY_CUDA(cudaMemcpyAsync(h->d_iq64_saved, h->d_iq64, sizeof(double) * h->n_q,
                                 cudaMemcpyDeviceToDevice, h->st),
                 "save curve");
    h->saved_bodies = h->cur;
    h->saved_ff = h->ff;
    h->saved_rsasa = h->rsasa;
    h->saved_ww = h->water_weight;
    h->saved_wi = h->water_index;
    h->saved_layout_version = h->layout_version;
    h->have_saved = true;
    RSX_TRY_CUDA(cudaStreamSynchronize(h->st), "commit");
    return ok();
}

rsx_status rsx_debye_revert(rsx_debye *h)
{
    RSX_TRY(begin_call(h));
    if (!h->computing)
        return fail(RSX_NO_INITIAL_CALC, "revert called before an initial call to calc");
    if (!h->have_saved)
        return ok(); // saxs_alg_cl_gpu_pt_wf.cpp:607-608
    h->ff = h->saved_ff;
    h->ff_on_device = false;
    h->rsasa = h->saved_rsasa;
    h->water_weight = h->saved_ww;
    h->water_index = h->saved_wi;
    if (h->layout_version != h->saved_layout_version) {
        // the body types changed since the checkpoint: rebuild from it
        RSX_TRY(full_calc(h, h->saved_bodies.data()));
        h->saved_layout_version = h->layout_version;
    } else {
        RSX_TRY_CUDA(cudaMemcpyAsync(h->d_pos, h->d_pos_saved, sizeof(float4) * h->n,
                                     cudaMemcpyDeviceToDevice, h->st),
                     "restore positions");
        RSX_TRY_CUDA(cudaMemcpyAsync(h->d_iq64, h->d_iq64_saved, sizeof(double) * h->n_q,
                                     cudaMemcpyDeviceToDevice, h->st),
                     "restore curve");
        RSX_TRY_CUDA(cudaMemcpyAsync(h->d_ff, h->ff.data(), sizeof(float) * h->ff.size(),
                                     cudaMemcpyHostToDevice, h->st),
                     "restore factors");
        h->ff_on_device = true;
        h->cur = h->saved_bodies;
        grow_extent(h, h->cur.data(), (unsigned)h->cur.size());
        RSX_TRY(upload_water(h));
        RSX_LAUNCH(launch_f64_to_f32(h->d_iq64, h->d_iq32, h->n_q, h->st), "curve f32");
        RSX_TRY_CUDA(cudaStreamSynchronize(h->st), "revert");
    }
    h->params_dirty = false;
    return ok();
}

rsx_status rsx_debye_curve_f64(rsx_debye *h, double *out_iq)
{
    RSX_TRY(begin_call(h));
    if (!h->computing)
        return fail(RSX_NO_INITIAL_CALC, "no curve computed yet");
    if (!out_iq)
        return fail(RSX_INVALID_ARG, "out is null");
    RSX_TRY_CUDA(cudaMemcpyAsync(h->h_iq64, h->d_iq64, sizeof(double) * h->n_q,
                                 cudaMemcpyDeviceToHost, h->st),
                 "read curve");
    RSX_TRY_CUDA(cudaStreamSynchronize(h->st), "read curve");
    std::memcpy(out_iq, h->h_iq64, sizeof(double) * h->n_q);
    return ok();
}

rsx_status rsx_debye_forward_resident(rsx_debye *h)
{
    RSX_TRY(begin_call(h));
    if (!h->computing)
        return fail(RSX_NO_INITIAL_CALC, "no bodies on the device yet");
    RSX_TRY(forward_device(h));
    return ok();
}

rsx_status rsx_debye_sync(rsx_debye *h)
{
    RSX_TRY(begin_call(h, false));
    RSX_TRY(finish_timing(h));
    RSX_TRY_CUDA(cudaStreamSynchronize(h->st), "sync");
    return ok();
}

void *rsx_debye_stream(rsx_debye *h) { return h ? (void *)h->st : nullptr; }

rsx_status rsx_debye_timing(rsx_debye *h, float *ms_pair_kernel, float *ms_call)
{
    if (!h)
        return fail(RSX_ALG_NOT_INITIALIZED, "null rsx_debye handle");
    if (!h->timing)
        return fail(RSX_ARGS_NOT_SET, "handle created without options.timing");
    if (ms_pair_kernel)
        *ms_pair_kernel = h->last_ms_kernel;
    if (ms_call)
        *ms_call = h->last_ms_call;
    return ok();
}

// Geometry of the adjoint's pair-function tables (pair_grid's nodes).  False
// when the tables would not fit the cap (the recurrence adjoint is used then).
static bool adjoint_table_geometry(const rsx_debye *h, int *nodes, float *step)
{
    double n = 0.0, st = 0.0;
    if (!pair_grid(h, &n, &st))
        return false;
    const double bytes = n * h->n_types * h->n_types * sizeof(float4) * (has_water(h) ? 4 : 1);
    if (!(n < 1e7) || bytes > 512.0 * 1024 * 1024)
        return false;
    *nodes = (int)n;
    *step = (float)st;
    return *step > 0.f;
}

static rsx_status backward_impl(rsx_debye *h, const float *dl_diq)
{
    if (!h->computing)
        return fail(RSX_NO_INITIAL_CALC, "backward called before an initial call to calc");
    if (!dl_diq)
        return fail(RSX_INVALID_ARG, "dL/dI is null");
    RSX_TRY_CUDA(cudaMemcpyAsync(h->d_lambda, dl_diq, sizeof(float) * h->n_q,
                                 cudaMemcpyHostToDevice, h->st),
                 "upload dL/dI");
    RSX_TRY_CUDA(cudaMemsetAsync(h->d_grad, 0, sizeof(double) * 3 * h->n, h->st), "zero grad");
    DebyeArgs a = debye_args(h);
    a.items = h->d_adj_items;
    a.n_items = (int)h->L.adj_items.size();
    a.lambda = h->d_lambda;
    a.grad = h->d_grad;
    int nodes = 0;
    float step = 0.f;
    const bool tables =
        h->pair_tables && h->n_types <= 32 && adjoint_table_geometry(h, &nodes, &step);
    if (tables) {
        RSX_TRY(ensure(&h->d_adj_tab, h->adj_tab_cap,
                       (size_t)nodes * h->n_types * h->n_types * (has_water(h) ? 4 : 1),
                       "adjoint tables"));
        a.adj_tab = h->d_adj_tab;
        a.adj_nodes = nodes;
        a.adj_h = step;
        a.adj_inv_h = 1.0f / step;
    }
    const unsigned type_mask = present_types(h);
    if (h->timing)
        RSX_TRY_CUDA(cudaEventRecord(h->ev_k0, h->st), "event");
    if (tables)
        RSX_LAUNCH(launch_adjoint_table(a, h->d_adj_tab, type_mask, has_water(h), h->st),
                   "adjoint kernels");
    else
        RSX_LAUNCH(launch_adjoint(a, slab_for(h), h->uniform, has_water(h), h->st),
                   "adjoint kernel");
    if (h->timing)
        RSX_TRY_CUDA(cudaEventRecord(h->ev_k1, h->st), "event");
    RSX_TRY_CUDA(cudaMemcpyAsync(h->h_grad, h->d_grad, sizeof(double) * 3 * h->n,
                                 cudaMemcpyDeviceToHost, h->st),
                 "read gradient");
    RSX_TRY(finish_timing(h));
    RSX_TRY_CUDA(cudaStreamSynchronize(h->st), "backward");
    return RSX_OK;
}

rsx_status rsx_debye_backward_f64(rsx_debye *h, const float *dl_diq, double *grad_xyz)
{
    RSX_TRY(begin_call(h));
    if (!grad_xyz)
        return fail(RSX_INVALID_ARG, "gradient output is null");
    // the host pointer may alias nothing of ours; dl_diq is pageable: copy first
    std::vector<float> lam(dl_diq ? dl_diq : nullptr, dl_diq ? dl_diq + h->n_q : nullptr);
    RSX_TRY(backward_impl(h, dl_diq ? lam.data() : nullptr));
    for (int s = 0; s < h->n; ++s) {
        const int c = h->L.perm[s];
        grad_xyz[3 * c + 0] = h->h_grad[3 * s + 0];
        grad_xyz[3 * c + 1] = h->h_grad[3 * s + 1];
        grad_xyz[3 * c + 2] = h->h_grad[3 * s + 2];
    }
    return ok();
}

rsx_status rsx_debye_backward(rsx_debye *h, const float *dl_diq, float *grad_xyz)
{
    RSX_TRY(begin_call(h));
    if (!grad_xyz)
        return fail(RSX_INVALID_ARG, "gradient output is null");
    std::vector<float> lam(dl_diq ? dl_diq : nullptr, dl_diq ? dl_diq + h->n_q : nullptr);
    RSX_TRY(backward_impl(h, dl_diq ? lam.data() : nullptr));
    for (int s = 0; s < h->n; ++s) {
        const int c = h->L.perm[s];
        grad_xyz[3 * c + 0] = (float)h->h_grad[3 * s + 0];
        grad_xyz[3 * c + 1] = (float)h->h_grad[3 * s + 1];
        grad_xyz[3 * c + 2] = (float)h->h_grad[3 * s + 2];
    }
    return ok();
}

rsx_status rsx_debye_chi2_backward(rsx_debye *h, const float *target, const float *sigma,
                                   double *chi2, float *grad_xyz)
{
    RSX_TRY(begin_call(h));
    if (!target || !sigma)
        return fail(RSX_INVALID_ARG, "target / sigma is null");
    std::vector<double> iq(h->n_q);
    RSX_TRY(rsx_debye_curve_f64(h, iq.data()));
    std::vector<float> lam(h->n_q);
    double c2 = 0.0;
    for (int k = 0; k < h->n_q; ++k) {
        const double s = sigma[k];
        if (!(s > 0.0))
            return fail(RSX_INVALID_ARG, "sigma must be positive");
        const double d = (iq[k] - target[k]) / s;
        c2 += d * d;
        lam[k] = (float)(2.0 * d / s);
    }
    if (chi2)
        *chi2 = c2;
    if (grad_xyz)
        RSX_TRY(rsx_debye_backward(h, lam.data(), grad_xyz));
    return ok();
}

rsx_status rsx_debye_tile_shape(rsx_debye *h, int *q_slab, int *pairs_per_step)
{
    if (!h)
        return fail(RSX_ALG_NOT_INITIALIZED, "null rsx_debye handle");
    if (q_slab)
        *q_slab = forward_slab(h);
    if (pairs_per_step)
        *pairs_per_step = h->pairs_per_step;
    return ok();
}

rsx_status rsx_debye_config(rsx_debye *h, int *q_slab, int *n_items, int *uniform_q)
{
    if (!h)
        return fail(RSX_ALG_NOT_INITIALIZED, "null rsx_debye handle");
    if (q_slab)
        *q_slab = forward_slab(h);
    if (n_items)
        *n_items = (int)h->L.items.size();
    if (uniform_q)
        *uniform_q = h->uniform ? 1 : 0;
    return ok();
}

rsx_status rsx_debug_layout(const rsx_body *bodies, int n_bodies, int n_factors, int max_items,
                            int min_adj_items, int *n_blocks, int *n_items, int *n_adj_items,
                            int *pairs_covered_ok)
{
    if ((!bodies && n_bodies > 0) || n_bodies < 0 || n_factors <= 0 || n_factors > kMaxTypes ||
        max_items <= 0)
        return fail(RSX_INVALID_ARG, "bad layout arguments");
    for (int i = 0; i < n_bodies; ++i)
        if (type_of(bodies[i]) >= (unsigned)n_factors)
            return fail(RSX_INVALID_ARG, "type out of range");
    Layout L;
    build_layout(L, bodies, n_bodies, n_factors, max_items, min_adj_items);
    if (n_blocks)
        *n_blocks = (int)L.blocks.size();
    if (n_items)
        *n_items = (int)L.items.size();
    if (n_adj_items)
        *n_adj_items = (int)L.adj_items.size();
    if (pairs_covered_ok) {
        // every unordered block pair (bi <= bj) must be covered exactly once
        // by each item list, and every block must hold one type only
        bool good = true;
        for (const auto &b : L.blocks)
            for (int s = b.start; s < b.start + b.len && good; ++s)
                good = L.types[L.perm[s]] == (unsigned)b.type;
        for (const auto *items : {&L.items, &L.adj_items}) {
            const int nb = (int)L.blocks.size();
            std::vector<int> seen((size_t)nb * nb, 0);
            for (const auto &it : *items) {
                if (it.bj_begin < it.bi || it.bj_end <= it.bj_begin)
                    good = false;
                for (int bj = it.bj_begin; bj < it.bj_end && good; ++bj) {
                    good = L.blocks[bj].type == L.blocks[it.bj_begin].type;
                    seen[(size_t)it.bi * nb + bj]++;
                }
            }
            for (int bi = 0; bi < nb; ++bi)
                for (int bj = 0; bj < nb; ++bj)
                    good = good && seen[(size_t)bi * nb + bj] == (bj >= bi ? 1 : 0);
        }
        *pairs_covered_ok = good ? 1 : 0;
    }
    return ok();
}

// ---- function-pointer ABI (host_debye.hpp:30) ------------------------------

static std::mutex g_fn_mu;

rsx_status rsx_calc_saxs_curve_status(const float *v_q, int n_q, const rsx_body *v_bodies,
                                      int n_bodies, const float *t_factors, int n_factors,
                                      float *out_v_Iq)
{
    if (!out_v_Iq || (n_bodies > 0 && !v_bodies))
        return fail(RSX_INVALID_ARG, "null pointer argument");
    std::lock_guard<std::mutex> lk(g_fn_mu);
    rsx_debye *h = nullptr;
    RSX_TRY(rsx_debye_create(v_q, n_q, t_factors, n_factors, n_bodies, nullptr, &h));
    rsx_status s = rsx_debye_calc(h, v_bodies, out_v_Iq);
    std::string msg = rsx_last_error();
    rsx_debye_destroy(h);
    if (s != RSX_OK)
        return fail(s, msg);
    return ok();
}

void rsx_calc_saxs_curve(const float *v_q, int n_q, const rsx_body *v_bodies, int n_bodies,
                         const float *t_factors, int n_factors, float *out_v_Iq)
{
    (void)rsx_calc_saxs_curve_status(v_q, n_q, v_bodies, n_bodies, t_factors, n_factors,
                                     out_v_Iq);
}

} // extern "C"
