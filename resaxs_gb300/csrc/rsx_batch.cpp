// Batched ensemble handle behind the C ABI: M conformations with their own
// body counts share one q grid and factor table.  Forward (and forward +
// chi^2 adjoint) of the whole ensemble run as one CUDA graph: H2D copy of the
// packed bodies, persistent pair kernels, per-member assembly, loss, D2H.
// No reference counterpart: the reference evaluates an ensemble one model at
// a time through i_saxs::calc_curve (calc_saxs/calc_saxs.hpp:611-624).
#include "rsx_batch_internal.h"
#include "rsx_host.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

using namespace rsx;

namespace {

unsigned btype(const rsx_body &b)
{
    unsigned t;
    std::memcpy(&t, &b.w, sizeof t);
    return t;
}

} // namespace

struct rsx_batch {
    int device = -1;
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int n_q = 0, n_types = 0, n_members = 0, n_total = 0;
    std::vector<float> q, ff;
    std::vector<int> sizes, offsets; // caller layout of the concatenated bodies
    bool uniform = false;
    float dq = 0.f;
    int small_theta = 0; // theta_level() the captured graphs were built with
    int q_slab = 64;
    int pairs_per_step = 2; // wide main slabs of 128 q and more: 2 or 4
    bool autotune = false, tuned = false;
    int sms = 152;

    // implicit water (forward only): weight 0 leaves it out; rsasa is kept in
    // caller order and staged per sorted slot with per-member sums
    float water_weight = 0.f;
    int water_index = 0;
    std::vector<float> rsasa;
    bool water_dirty = false;
    float *d_rsasa = nullptr;       // [n_total] per sorted slot
    double *d_water_sums = nullptr; // [M][T] by type, [M] of rsasa^2, [M] of rsasa

    // layout (rebuilt when any body type changes)
    bool have_layout = false;
    std::vector<unsigned> types;     // caller order
    std::vector<int> perm;           // sorted slot -> caller index
    std::vector<BlockDesc> blocks;
    std::vector<PairItem> items;     // forward
    std::vector<PairItem> adj_items; // adjoint
    std::vector<int> order, adj_order;
    std::vector<int2> item_range;
    std::vector<int> type_count;     // [M][T]

    // device
    float4 *d_pos = nullptr;
    float *d_ff = nullptr, *d_q = nullptr;
    BlockDesc *d_blocks = nullptr;
    PairItem *d_items = nullptr, *d_adj_items = nullptr;
    int *d_order = nullptr, *d_adj_order = nullptr;
    int2 *d_range = nullptr;
    int *d_type_count = nullptr;
    double *d_partial = nullptr;
    double *d_iq64 = nullptr;
    float *d_iq32 = nullptr;
    float *d_target = nullptr, *d_sigma = nullptr, *d_lambda = nullptr;
    double *d_chi2 = nullptr, *d_grad = nullptr;
    int *d_counter = nullptr; // [4]
    // pinned
    float4 *h_pos = nullptr;
    float *h_iq = nullptr;
    double *h_chi2 = nullptr, *h_grad = nullptr;
    bool have_targets = false;

    // adjoint through tabulated pair functions: the node count is a capacity
    // fixed in the captured graphs (0: the recurrence adjoint); the step of a
    // pass travels through h_adj_geom -> d_adj_geom ([h, 1/h]) at replay
    bool pair_tables = true; // 0: the recurrence adjoint
    float4 *d_adj_tab = nullptr;
    int adj_nodes = 0;
    float *h_adj_geom = nullptr, *d_adj_geom = nullptr;
    double q_max = 0.0;

    cudaGraphExec_t g_fwd = nullptr, g_fwd_adj = nullptr;
    int fwd_grid = 0, adj_grid = 0, adj_table_grid = 0;
    float last_ms = 0.f;
};

namespace {

void drop_graphs(rsx_batch *h)
{
    if (h->g_fwd)
        cudaGraphExecDestroy(h->g_fwd);
    if (h->g_fwd_adj)
        cudaGraphExecDestroy(h->g_fwd_adj);
    h->g_fwd = h->g_fwd_adj = nullptr;
}

void free_layout_buffers(rsx_batch *h)
{
    void *p[] = {h->d_blocks, h->d_items, h->d_adj_items, h->d_order, h->d_adj_order,
                 h->d_range, h->d_type_count, h->d_partial};
    for (void *x : p)
        dev_free(x);
    h->d_blocks = nullptr;
    h->d_items = h->d_adj_items = nullptr;
    h->d_order = h->d_adj_order = nullptr;
    h->d_range = nullptr;
    h->d_type_count = nullptr;
    h->d_partial = nullptr;
}

rsx_status batch_release(rsx_batch *h)
{
    if (!h)
        return RSX_OK;
    DeviceGuard g(h->device);
    if (h->st)
        cudaStreamSynchronize(h->st);
    drop_graphs(h);
    free_layout_buffers(h);
    void *dev[] = {h->d_pos,    h->d_ff,     h->d_q,      h->d_iq64,    h->d_iq32,
                   h->d_target, h->d_sigma, h->d_lambda, h->d_chi2,    h->d_grad,
                   h->d_counter, h->d_adj_tab, h->d_adj_geom, h->d_rsasa, h->d_water_sums};
    for (void *x : dev)
        dev_free(x);
    void *pin[] = {h->h_pos, h->h_iq, h->h_chi2, h->h_grad, h->h_adj_geom};
    for (void *x : pin)
        host_free_pinned(x);
    if (h->e0)
        cudaEventDestroy(h->e0);
    if (h->e1)
        cudaEventDestroy(h->e1);
    if (h->st)
        cudaStreamDestroy(h->st);
    delete h;
    return RSX_OK;
}

std::vector<PairItem> member_items(const std::vector<BlockDesc> &blocks, int b0, int b1,
                                   int jchunk, int member)
{
    std::vector<PairItem> items;
    for (int bi = b0; bi < b1; ++bi) {
        int bj = bi;
        while (bj < b1) {
            const int t = blocks[bj].type;
            int end = bj;
            while (end < b1 && blocks[end].type == t && end - bj < jchunk)
                ++end;
            items.push_back(PairItem{bi, bj, end, member});
            bj = end;
        }
    }
    return items;
}

long long item_work(const std::vector<BlockDesc> &blocks, const PairItem &it)
{
    long long j = 0;
    for (int b = it.bj_begin; b < it.bj_end; ++b)
        j += blocks[b].len;
    return (long long)blocks[it.bi].len * j;
}

rsx_status build_batch_layout(rsx_batch *h, const rsx_body *bodies)
{
    const int T = h->n_types, M = h->n_members;
    h->types.resize(h->n_total);
    for (int i = 0; i < h->n_total; ++i)
        h->types[i] = btype(bodies[i]);
    h->perm.resize(h->n_total);
    h->blocks.clear();
    h->items.clear();
    h->adj_items.clear();
    h->item_range.assign(M, int2{0, 0});
    h->type_count.assign((size_t)M * T, 0);
    std::vector<std::pair<int, int>> member_blocks(M);
    for (int m = 0; m < M; ++m) {
        const int off = h->offsets[m], n = h->sizes[m];
        int *cnt = &h->type_count[(size_t)m * T];
        for (int i = 0; i < n; ++i)
            cnt[h->types[off + i]]++;
        std::vector<int> start(T + 1, 0);
        for (int t = 0; t < T; ++t)
            start[t + 1] = start[t] + cnt[t];
        std::vector<int> fill(start.begin(), start.end() - 1);
        for (int i = 0; i < n; ++i)
            h->perm[off + fill[h->types[off + i]]++] = off + i;
        const int b0 = (int)h->blocks.size();
        for (int t = 0; t < T; ++t)
            for (int s = start[t]; s < start[t + 1]; s += kBlockAtoms)
                h->blocks.push_back(
                    BlockDesc{off + s, std::min(kBlockAtoms, start[t + 1] - s), t, 0});
        member_blocks[m] = {b0, (int)h->blocks.size()};
    }
    // forward items: J runs grouped so the total stays below ~64k items
    // (scratch = items * n_q doubles); adjoint items: single J blocks
    int jchunk = 1;
    for (;;) {
        long long total = 0;
        for (int m = 0; m < M; ++m) {
            const long long nb = member_blocks[m].second - member_blocks[m].first;
            total += nb * (nb + 1) / 2 / jchunk + nb * T;
        }
        if (total <= 65536 || jchunk >= 1024)
            break;
        jchunk *= 2;
    }
    for (int m = 0; m < M; ++m) {
        const int x = (int)h->items.size();
        auto it = member_items(h->blocks, member_blocks[m].first, member_blocks[m].second,
                               jchunk, m);
        h->items.insert(h->items.end(), it.begin(), it.end());
        h->item_range[m] = int2{x, (int)h->items.size()};
        auto ia = member_items(h->blocks, member_blocks[m].first, member_blocks[m].second, 1, m);
        h->adj_items.insert(h->adj_items.end(), ia.begin(), ia.end());
    }
    auto by_work = [&](const std::vector<PairItem> &items, std::vector<int> &order) {
        order.resize(items.size());
        std::iota(order.begin(), order.end(), 0);
        std::vector<long long> w(items.size());
        for (size_t i = 0; i < items.size(); ++i)
            w[i] = item_work(h->blocks, items[i]);
        std::stable_sort(order.begin(), order.end(),
                         [&](int a, int b) { return w[a] > w[b]; });
    };
    by_work(h->items, h->order);
    by_work(h->adj_items, h->adj_order);

    free_layout_buffers(h);
    const size_t nb = std::max<size_t>(h->blocks.size(), 1);
    const size_t ni = std::max<size_t>(h->items.size(), 1);
    const size_t na = std::max<size_t>(h->adj_items.size(), 1);
    RSX_TRY(dev_alloc((void **)&h->d_blocks, sizeof(BlockDesc) * nb, "batch blocks"));
    RSX_TRY(dev_alloc((void **)&h->d_items, sizeof(PairItem) * ni, "batch items"));
    RSX_TRY(dev_alloc((void **)&h->d_adj_items, sizeof(PairItem) * na, "batch adjoint items"));
    RSX_TRY(dev_alloc((void **)&h->d_order, sizeof(int) * ni, "batch order"));
    RSX_TRY(dev_alloc((void **)&h->d_adj_order, sizeof(int) * na, "batch adjoint order"));
    RSX_TRY(dev_alloc((void **)&h->d_range, sizeof(int2) * std::max(M, 1), "member ranges"));
    RSX_TRY(dev_alloc((void **)&h->d_type_count, sizeof(int) * std::max(M * T, 1), "type counts"));
    RSX_TRY(dev_alloc((void **)&h->d_partial, sizeof(double) * ni * h->n_q, "batch partials"));
    auto up = [&](void *dst, const void *src, size_t bytes, const char *what) -> rsx_status {
        if (bytes == 0)
            return RSX_OK;
        RSX_TRY_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, h->st), what);
        return RSX_OK;
    };
    RSX_TRY(up(h->d_blocks, h->blocks.data(), sizeof(BlockDesc) * h->blocks.size(), "blocks"));
    RSX_TRY(up(h->d_items, h->items.data(), sizeof(PairItem) * h->items.size(), "items"));
    RSX_TRY(up(h->d_adj_items, h->adj_items.data(), sizeof(PairItem) * h->adj_items.size(),
               "adjoint items"));
    RSX_TRY(up(h->d_order, h->order.data(), sizeof(int) * h->order.size(), "order"));
    RSX_TRY(up(h->d_adj_order, h->adj_order.data(), sizeof(int) * h->adj_order.size(),
               "adjoint order"));
    RSX_TRY(up(h->d_range, h->item_range.data(), sizeof(int2) * M, "ranges"));
    RSX_TRY(up(h->d_type_count, h->type_count.data(), sizeof(int) * h->type_count.size(),
               "counts"));
    RSX_TRY_CUDA(cudaStreamSynchronize(h->st), "batch layout");
    h->have_layout = true;
    h->water_dirty = true; // new slot order
    drop_graphs(h);
    return RSX_OK;
}

bool has_water(const rsx_batch *h) { return h->water_weight != 0.f; }

// rsasa per sorted slot and, per member, its sums by type, of squares and in
// total (summed in caller order, as the single-structure handle does).
rsx_status upload_water(rsx_batch *h)
{
    const int T = h->n_types, M = h->n_members;
    std::vector<float> sorted((size_t)std::max(h->n_total, 1), 0.f);
    std::vector<double> sums((size_t)M * T + 2 * (size_t)M, 0.0);
    for (int m = 0; m < M; ++m) {
        const int end = h->offsets[m] + h->sizes[m];
        for (int i = h->offsets[m]; i < end; ++i) {
            const double r = h->rsasa[i];
            sums[(size_t)m * T + h->types[i]] += r;
            sums[(size_t)M * T + m] += r * r;
            sums[(size_t)M * T + M + m] += r;
        }
    }
    for (int s = 0; s < h->n_total; ++s)
        sorted[s] = h->rsasa[h->perm[s]];
    RSX_TRY_CUDA(cudaMemcpyAsync(h->d_rsasa, sorted.data(), sizeof(float) * sorted.size(),
                                 cudaMemcpyHostToDevice, h->st),
                 "upload rsasa");
    if (!sums.empty())
        RSX_TRY_CUDA(cudaMemcpyAsync(h->d_water_sums, sums.data(), sizeof(double) * sums.size(),
                                     cudaMemcpyHostToDevice, h->st),
                     "upload rsasa sums");
    RSX_TRY_CUDA(cudaStreamSynchronize(h->st), "upload water");
    h->water_dirty = false;
    return RSX_OK;
}

// The q slab the forward kernels run with: water keeps two accumulator sets
// per thread, so its slabs stop at 16 q (128 q on the wide uniform path).
int water_slab(const rsx_batch *h, int q_slab)
{
    if (!has_water(h) || (h->uniform && q_slab >= 64))
        return q_slab;
    return q_slab >= 16 ? 16 : 8;
}

DebyeArgs batch_args(rsx_batch *h, bool adjoint)
{
    DebyeArgs a{};
    a.pos = h->d_pos;
    a.ff = h->d_ff;
    a.q = h->d_q;
    a.blocks = h->d_blocks;
    a.items = adjoint ? h->d_adj_items : h->d_items;
    a.partial = h->d_partial;
    a.n = h->n_total;
    a.n_q = h->n_q;
    a.n_types = h->n_types;
    a.n_items = (int)(adjoint ? h->adj_items.size() : h->items.size());
    a.dq = h->dq;
    a.small_theta = h->small_theta;
    a.pairs4 = h->pairs_per_step == 4 ? 1 : 0;
    a.lambda = h->d_lambda;
    a.grad = h->d_grad;
    if (!adjoint && has_water(h)) {
        a.rsasa = h->d_rsasa;
        a.water_weight = h->water_weight;
        a.water_index = h->water_index;
    }
    return a;
}

// Enqueues one ensemble pass on the stream (used for capture).
rsx_status enqueue_pass(rsx_batch *h, bool with_adjoint, int q_slab)
{
    const size_t nbody = (size_t)std::max(h->n_total, 1);
    RSX_TRY_CUDA(cudaMemcpyAsync(h->d_pos, h->h_pos, sizeof(float4) * nbody,
                                 cudaMemcpyHostToDevice, h->st),
                 "batch bodies");
    RSX_TRY_CUDA(cudaMemsetAsync(h->d_counter, 0, sizeof(int) * 4, h->st), "counters");
    const DebyeArgs a = batch_args(h, false);
    const int n_items = (int)h->items.size();
    const bool water = has_water(h);
    const bool wide = h->uniform && q_slab >= 64;
    // the wide launches of a grid from q = 0 (with q[1] == dq) run on q[1..]
    // (past_q0)
    const bool q0_free = wide && h->n_q > 1 && h->q[0] == 0.f && h->q[1] == h->dq;
    const DebyeArgs aw = q0_free ? past_q0(a, n_items) : a;
    // q_slab 192 without water and with two pairs per step: chained slabs
    if (wide && !water && q_slab >= 192 && h->pairs_per_step != 4)
        RSX_TRY_CUDA(launch_batch_forward_chain(aw, h->d_order, n_items, h->d_counter, h->sms,
                                                h->st),
                     "batch forward");
    else if (wide)
        RSX_TRY_CUDA(launch_batch_forward_wide(aw, h->d_order, n_items, q_slab, h->d_counter,
                                               h->sms, h->st, water),
                     "batch forward");
    const int slab = water_slab(h, q_slab);
    const int full = wide ? 0 : h->n_q / slab, rest = wide ? 0 : h->n_q - full * slab;
    if (full > 0)
        RSX_TRY_CUDA(launch_batch_forward(a, h->d_order, n_items, slab, full, 0, h->uniform,
                                          h->d_counter + 0, h->fwd_grid, h->st, water),
                     "batch forward");
    if (rest > 0) {
        const int tail = rest <= 8 ? 8 : (rest <= 16 ? 16 : 32);
        const int n_tail = (rest + tail - 1) / tail;
        const int grid = batch_forward_grid(tail, h->uniform, h->sms, water);
        RSX_TRY_CUDA(launch_batch_forward(a, h->d_order, n_items, tail, n_tail, full * slab,
                                          h->uniform, h->d_counter + 1, grid, h->st, water),
                     "batch forward tail");
    }
    BatchAssembleArgs b{};
    b.partial = h->d_partial;
    b.ff = h->d_ff;
    b.q = h->d_q;
    b.type_count = h->d_type_count;
    b.item_range = h->d_range;
    b.n_q = h->n_q;
    b.n_types = h->n_types;
    b.n_items = n_items;
    b.n_members = h->n_members;
    b.iq64 = h->d_iq64;
    b.iq32 = h->d_iq32;
    if (water) {
        const size_t MT = (size_t)h->n_members * h->n_types;
        b.rsasa_sum = h->d_water_sums;
        b.rsasa_sq = h->d_water_sums + MT;
        b.rsasa_tot = h->d_water_sums + MT + h->n_members;
        b.water_weight = h->water_weight;
        b.water_index = h->water_index;
        b.has_water = 1;
    }
    RSX_TRY_CUDA(launch_batch_assemble(b, h->st), "batch assemble");
    if (with_adjoint) {
        BatchLossArgs l{};
        l.iq64 = h->d_iq64;
        l.target = h->d_target;
        l.sigma = h->d_sigma;
        l.n_q = h->n_q;
        l.n_members = h->n_members;
        l.lambda = h->d_lambda;
        l.chi2 = h->d_chi2;
        RSX_TRY_CUDA(launch_batch_loss(l, h->st), "batch loss");
        RSX_TRY_CUDA(cudaMemsetAsync(h->d_grad, 0, sizeof(double) * 3 * nbody, h->st), "grad");
        DebyeArgs g = batch_args(h, true);
        if (h->adj_nodes > 0) {
            g.adj_tab = h->d_adj_tab;
            g.adj_nodes = h->adj_nodes;
            g.adj_geom = h->d_adj_geom;
            RSX_TRY_CUDA(cudaMemcpyAsync(h->d_adj_geom, h->h_adj_geom, sizeof(float) * 2,
                                         cudaMemcpyHostToDevice, h->st),
                         "adjoint table step");
            const unsigned mask = h->n_types >= 32 ? 0xffffffffu : (1u << h->n_types) - 1u;
            RSX_TRY_CUDA(launch_adjoint_tables(g, h->d_adj_tab, mask, h->n_members, h->st),
                         "adjoint tables");
            RSX_TRY_CUDA(launch_batch_adjoint_table(g, h->d_adj_order, (int)h->adj_items.size(),
                                                    h->d_counter + 2, h->adj_table_grid, h->st),
                         "batch adjoint");
        } else {
            RSX_TRY_CUDA(launch_batch_adjoint(g, h->d_adj_order, (int)h->adj_items.size(),
                                              q_slab, h->uniform, h->d_counter + 2, h->adj_grid,
                                              h->st),
                         "batch adjoint");
        }
        RSX_TRY_CUDA(cudaMemcpyAsync(h->h_chi2, h->d_chi2, sizeof(double) * h->n_members,
                                     cudaMemcpyDeviceToHost, h->st),
                     "read chi2");
        RSX_TRY_CUDA(cudaMemcpyAsync(h->h_grad, h->d_grad, sizeof(double) * 3 * nbody,
                                     cudaMemcpyDeviceToHost, h->st),
                     "read grad");
    }
    RSX_TRY_CUDA(cudaMemcpyAsync(h->h_iq, h->d_iq32, sizeof(float) * h->n_members * h->n_q,
                                 cudaMemcpyDeviceToHost, h->st),
                 "read curves");
    return RSX_OK;
}

rsx_status capture(rsx_batch *h, bool with_adjoint, cudaGraphExec_t *out)
{
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device);
    h->sms = sms;
    h->fwd_grid = batch_forward_grid(water_slab(h, h->q_slab), h->uniform, sms,
                                     has_water(h) && !(h->uniform && h->q_slab >= 64));
    h->adj_grid = batch_adjoint_grid(h->q_slab, h->uniform, h->n_q, sms);
    h->adj_table_grid = batch_adjoint_table_grid(sms);
    RSX_TRY_CUDA(cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal),
                 "begin capture");
    rsx_status s = enqueue_pass(h, with_adjoint, h->q_slab);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(h->st, &g);
    if (s != RSX_OK) {
        if (g)
            cudaGraphDestroy(g);
        return s;
    }
    if (e != cudaSuccess)
        return cuda_status(e, "end capture");
    e = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess)
        return cuda_status(e, "instantiate graph");
    return RSX_OK;
}

rsx_status stage_bodies(rsx_batch *h, const rsx_body *bodies)
{
    // One sequential pass: factor indices, whether the type layout is the one
    // the graphs were built for, and each member's bounding box (min and max
    // of floats are exact; the diagonal is formed in double).
    bool same = h->have_layout;
    double worst = 0.0;
    for (int m = 0; m < h->n_members; ++m) {
        float lo[3] = {3.4e38f, 3.4e38f, 3.4e38f}, hi[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
        const int end = h->offsets[m] + h->sizes[m];
        for (int i = h->offsets[m]; i < end; ++i) {
            const rsx_body &b = bodies[i];
            const unsigned t = btype(b);
            if (t >= (unsigned)h->n_types)
                return fail(RSX_INVALID_ARG,
                            "body " + std::to_string(i) + " has a factor index >= n_factors");
            same = same && t == h->types[i];
            lo[0] = std::min(lo[0], b.x);
            hi[0] = std::max(hi[0], b.x);
            lo[1] = std::min(lo[1], b.y);
            hi[1] = std::max(hi[1], b.y);
            lo[2] = std::min(lo[2], b.z);
            hi[2] = std::max(hi[2], b.z);
        }
        if (h->sizes[m] > 1) {
            double d2 = 0.0;
            for (int d = 0; d < 3; ++d)
                d2 += ((double)hi[d] - lo[d]) * ((double)hi[d] - lo[d]);
            worst = std::max(worst, std::sqrt(d2));
        }
    }
    if (!same)
        RSX_TRY(build_batch_layout(h, bodies));
    RSX_TRY_CUDA(cudaStreamSynchronize(h->st), "batch staging");
    for (int s = 0; s < h->n_total; ++s) {
        const rsx_body &b = bodies[h->perm[s]];
        h->h_pos[s] = make_float4(b.x, b.y, b.z, b.w);
    }
    // Adjoint tables: nodes for the widest member with q_max h <= 0.05.  The
    // capacity grows (with headroom) only when a pass needs more nodes; the
    // graphs are captured again then.  Past 1 GB the recurrence adjoint runs.
    {
        const double r_max = worst * 1.0001 + 1e-3;
        const double need = std::max(16.0, std::ceil(r_max * h->q_max / 0.05) + 2.0);
        if (h->pair_tables && need > h->adj_nodes) {
            const double nodes = std::ceil(need * 1.25);
            const double bytes = nodes * h->n_types * h->n_types * (double)h->n_members *
                                 sizeof(float4);
            dev_free(h->d_adj_tab);
            h->d_adj_tab = nullptr;
            const int before = h->adj_nodes;
            h->adj_nodes = 0;
            if (bytes <= 1024.0 * 1024 * 1024 && h->n_types <= 32 && h->n_members <= 65535 &&
                dev_alloc((void **)&h->d_adj_tab, (size_t)bytes, "adjoint tables") == RSX_OK)
                h->adj_nodes = (int)nodes;
            if (h->adj_nodes != before)
                drop_graphs(h);
        }
        if (h->adj_nodes > 0) {
            const double step = r_max / (h->adj_nodes - 2);
            h->h_adj_geom[0] = (float)step;
            h->h_adj_geom[1] = (float)(1.0 / (float)step);
        }
    }
    // theta_level() of the widest member selects the kernel instantiations
    // (the reduction-free seeds give the same results bit for bit).  It is a
    // kernel argument of the captured graphs, so they are captured again when
    // it changes.
    const int small = theta_level(h->uniform, (double)h->dq, worst);
    if (small != h->small_theta) {
        drop_graphs(h);
        h->small_theta = small;
    }
    return RSX_OK;
}

rsx_status run_graph(rsx_batch *h, cudaGraphExec_t g)
{
    RSX_TRY_CUDA(cudaEventRecord(h->e0, h->st), "event");
    if (inject_launch_fault())
        return fail(RSX_INJECTED_FAULT, "injected launch fault: batch graph");
    RSX_TRY_CUDA(cudaGraphLaunch(g, h->st), "graph launch");
    RSX_TRY_CUDA(cudaEventRecord(h->e1, h->st), "event");
    RSX_TRY_CUDA(cudaStreamSynchronize(h->st), "batch pass");
    cudaEventElapsedTime(&h->last_ms, h->e0, h->e1);
    return RSX_OK;
}

// Times one forward pass with each candidate tile shape (q-slab plan, and
// for the wide slabs of 128 q and more the pairs stepped together; encoded as
// q_slab + 1000 * (pairs_per_step == 4)) and keeps the fastest.
rsx_status tune(rsx_batch *h)
{
    const int candidates[] = {32, 64, 128, 1128, 192, 1192};
    float best = 1e30f;
    int best_qs = h->q_slab, best_pp = h->pairs_per_step;
    for (int c : candidates) {
        const int qs = c % 1000;
        if (qs >= 64 && !h->uniform)
            continue;
        if (qs == 192 && h->n_q < 192)
            continue;
        // the water kernels step two pairs and stop at 128 q per slab
        if (has_water(h) && (c >= 1000 || qs == 192))
            continue;
        h->q_slab = qs;
        h->pairs_per_step = c >= 1000 ? 4 : 2;
        cudaGraphExec_t g = nullptr;
        RSX_TRY(capture(h, false, &g));
        rsx_status s = run_graph(h, g); // warm
        if (s == RSX_OK)
            s = run_graph(h, g);
        cudaGraphExecDestroy(g);
        RSX_TRY(s);
        if (h->last_ms < best) {
            best = h->last_ms;
            best_qs = qs;
            best_pp = h->pairs_per_step;
        }
    }
    h->q_slab = best_qs;
    h->pairs_per_step = best_pp;
    h->tuned = true;
    return RSX_OK;
}

} // namespace

extern "C" {

rsx_status rsx_batch_create(const float *q, int n_q, const float *t_factors, int n_factors,
                            const int *member_sizes, int n_members,
                            const rsx_debye_options *opts, rsx_batch **out)
{
    if (!out)
        return fail(RSX_INVALID_ARG, "out handle pointer is null");
    *out = nullptr;
    if (!q || !t_factors || n_q <= 0 || n_factors <= 0 || n_members < 0 ||
        (n_members > 0 && !member_sizes))
        return fail(RSX_INVALID_ARG, "q, factors and member sizes must be non-null / positive");
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
    long long total = 0;
    for (int m = 0; m < n_members; ++m) {
        if (member_sizes[m] < 0)
            return fail(RSX_INVALID_ARG, "negative member size");
        total += member_sizes[m];
    }
    if (total > (1LL << 30))
        return fail(RSX_INVALID_ARG, "too many bodies");
    int dev = -1;
    RSX_TRY(select_device(o.device, &dev));
    DeviceGuard guard(dev);
    cudaSetDevice(dev);
    rsx_batch *h = new rsx_batch();
    h->device = dev;
    h->n_q = n_q;
    h->n_types = n_factors;
    h->n_members = n_members;
    h->n_total = (int)total;
    h->q.assign(q, q + n_q);
    for (int k = 0; k < n_q; ++k)
        h->q_max = std::max(h->q_max, std::fabs((double)q[k]));
    h->ff.assign(t_factors, t_factors + (size_t)n_q * n_factors);
    h->sizes.assign(member_sizes, member_sizes + n_members);
    h->offsets.resize(n_members);
    for (int m = 0, off = 0; m < n_members; ++m) {
        h->offsets[m] = off;
        off += member_sizes[m];
    }
    // uniform grid check as in the single-structure handle
    h->uniform = !o.force_general_q;
    if (n_q > 1 && h->uniform) {
        const double q0 = q[0], step = ((double)q[n_q - 1] - q0) / (n_q - 1);
        for (int k = 0; k < n_q && h->uniform; ++k)
            h->uniform = std::fabs((double)q[k] - (q0 + k * step)) <= 4e-7 * std::fabs((double)q[k]) + 1e-30;
        h->dq = (float)step;
    }
    h->q_slab = o.q_slab ? o.q_slab : (h->uniform && n_q >= 64 ? 192 : 32);
    if (!h->uniform && h->q_slab > 32)
        h->q_slab = 32;
    h->pairs_per_step = o.pairs_per_step ? o.pairs_per_step : 2;
    h->autotune = o.autotune != 0 && o.q_slab == 0 && o.pairs_per_step == 0;
    h->pair_tables = o.no_pair_tables == 0;
    auto bail = [&](rsx_status s) {
        batch_release(h);
        return s;
    };
    cudaError_t e = cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking);
    if (e == cudaSuccess)
        e = cudaEventCreate(&h->e0);
    if (e == cudaSuccess)
        e = cudaEventCreate(&h->e1);
    if (e != cudaSuccess)
        return bail(cuda_status(e, "batch stream"));
    const size_t nb = (size_t)std::max(h->n_total, 1), M = (size_t)std::max(n_members, 1);
    rsx_status s;
#define RSX_A(p, bytes, what)                                                              \
    if ((s = dev_alloc((void **)&(p), (bytes), what)) != RSX_OK)                           \
        return bail(s);
#define RSX_P(p, bytes, what)                                                              \
    if ((s = host_alloc_pinned((void **)&(p), (bytes), what)) != RSX_OK)                   \
        return bail(s);
    RSX_A(h->d_pos, sizeof(float4) * nb, "batch bodies");
    RSX_A(h->d_ff, sizeof(float) * h->ff.size(), "factors");
    RSX_A(h->d_q, sizeof(float) * n_q, "q");
    RSX_A(h->d_iq64, sizeof(double) * M * n_q, "curves");
    RSX_A(h->d_iq32, sizeof(float) * M * n_q, "curves f32");
    RSX_A(h->d_target, sizeof(float) * M * n_q, "targets");
    RSX_A(h->d_sigma, sizeof(float) * M * n_q, "sigmas");
    RSX_A(h->d_lambda, sizeof(float) * M * n_q, "dL/dI");
    RSX_A(h->d_chi2, sizeof(double) * M, "chi2");
    RSX_A(h->d_grad, sizeof(double) * 3 * nb, "gradient");
    RSX_A(h->d_counter, sizeof(int) * 4, "work counters");
    RSX_A(h->d_adj_geom, sizeof(float) * 2, "adjoint table step");
    RSX_P(h->h_adj_geom, sizeof(float) * 2, "pinned adjoint table step");
    RSX_P(h->h_pos, sizeof(float4) * nb, "pinned bodies");
    RSX_P(h->h_iq, sizeof(float) * M * n_q, "pinned curves");
    RSX_P(h->h_chi2, sizeof(double) * M, "pinned chi2");
    RSX_P(h->h_grad, sizeof(double) * 3 * nb, "pinned gradient");
#undef RSX_A
#undef RSX_P
    e = cudaMemcpyAsync(h->d_q, h->q.data(), sizeof(float) * n_q, cudaMemcpyHostToDevice, h->st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(h->d_ff, h->ff.data(), sizeof(float) * h->ff.size(),
                            cudaMemcpyHostToDevice, h->st);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(h->st);
    if (e != cudaSuccess)
        return bail(cuda_status(e, "batch initialisation"));
    *out = h;
    return ok();
}

rsx_status rsx_batch_destroy(rsx_batch *h)
{
    batch_release(h);
    return ok();
}

rsx_status rsx_batch_forward(rsx_batch *h, const rsx_body *bodies, float *out_iq)
{
    if (!h)
        return fail(RSX_ALG_NOT_INITIALIZED, "null rsx_batch handle");
    if ((!bodies && h->n_total > 0) || !out_iq)
        return fail(RSX_INVALID_ARG, "null bodies / output");
    RSX_TRY_CUDA(cudaSetDevice(h->device), "cudaSetDevice");
    RSX_TRY(stage_bodies(h, bodies));
    if (has_water(h) && h->water_dirty)
        RSX_TRY(upload_water(h));
    if (h->autotune && !h->tuned) {
        drop_graphs(h);
        RSX_TRY(tune(h));
    }
    if (!h->g_fwd)
        RSX_TRY(capture(h, false, &h->g_fwd));
    RSX_TRY(run_graph(h, h->g_fwd));
    std::memcpy(out_iq, h->h_iq, sizeof(float) * h->n_members * h->n_q);
    return ok();
}

rsx_status rsx_batch_set_targets(rsx_batch *h, const float *targets, const float *sigma)
{
    if (!h)
        return fail(RSX_ALG_NOT_INITIALIZED, "null rsx_batch handle");
    if (!targets || !sigma)
        return fail(RSX_INVALID_ARG, "targets / sigma are null");
    const size_t n = (size_t)h->n_members * h->n_q;
    for (size_t i = 0; i < n; ++i)
        if (!(sigma[i] > 0.f) || !std::isfinite(sigma[i]) || !std::isfinite(targets[i]))
            return fail(RSX_INVALID_ARG, "sigma must be positive and targets finite");
    RSX_TRY_CUDA(cudaSetDevice(h->device), "cudaSetDevice");
    RSX_TRY_CUDA(cudaMemcpyAsync(h->d_target, targets, sizeof(float) * n, cudaMemcpyHostToDevice,
                                 h->st),
                 "targets");
    RSX_TRY_CUDA(cudaMemcpyAsync(h->d_sigma, sigma, sizeof(float) * n, cudaMemcpyHostToDevice,
                                 h->st),
                 "sigmas");
    RSX_TRY_CUDA(cudaStreamSynchronize(h->st), "targets");
    h->have_targets = true;
    return ok();
}

rsx_status rsx_batch_forward_chi2_backward(rsx_batch *h, const rsx_body *bodies, float *out_iq,
                                           double *chi2, float *grad_xyz)
{
    if (!h)
        return fail(RSX_ALG_NOT_INITIALIZED, "null rsx_batch handle");
    if (!h->have_targets)
        return fail(RSX_ARGS_NOT_SET, "rsx_batch_set_targets was not called");
    if (has_water(h))
        return fail(RSX_NOT_SUPPORTED, "the batched adjoint has no implicit water term");
    if ((!bodies && h->n_total > 0))
        return fail(RSX_INVALID_ARG, "null bodies");
    RSX_TRY_CUDA(cudaSetDevice(h->device), "cudaSetDevice");
    RSX_TRY(stage_bodies(h, bodies));
    if (!h->g_fwd_adj)
        RSX_TRY(capture(h, true, &h->g_fwd_adj));
    RSX_TRY(run_graph(h, h->g_fwd_adj));
    if (out_iq)
        std::memcpy(out_iq, h->h_iq, sizeof(float) * h->n_members * h->n_q);
    if (chi2)
        std::memcpy(chi2, h->h_chi2, sizeof(double) * h->n_members);
    if (grad_xyz)
        for (int s = 0; s < h->n_total; ++s) {
            const int c = h->perm[s];
            grad_xyz[3 * c + 0] = (float)h->h_grad[3 * s + 0];
            grad_xyz[3 * c + 1] = (float)h->h_grad[3 * s + 1];
            grad_xyz[3 * c + 2] = (float)h->h_grad[3 * s + 2];
        }
    return ok();
}

rsx_status rsx_batch_set_factors(rsx_batch *h, const float *t_factors, int n_factors)
{
    if (!h)
        return fail(RSX_ALG_NOT_INITIALIZED, "null rsx_batch handle");
    if (!t_factors || n_factors != h->n_types)
        return fail(RSX_INVALID_ARG, "factor table must have the handle's n_factors columns");
    RSX_TRY_CUDA(cudaSetDevice(h->device), "cudaSetDevice");
    h->ff.assign(t_factors, t_factors + (size_t)h->n_q * n_factors);
    // the captured graphs read the table from d_ff
    RSX_TRY_CUDA(cudaMemcpyAsync(h->d_ff, h->ff.data(), sizeof(float) * h->ff.size(),
                                 cudaMemcpyHostToDevice, h->st),
                 "factors");
    RSX_TRY_CUDA(cudaStreamSynchronize(h->st), "factors");
    return ok();
}

rsx_status rsx_batch_set_water(rsx_batch *h, float weight, int water_index, const float *rsasa)
{
    if (!h)
        return fail(RSX_ALG_NOT_INITIALIZED, "null rsx_batch handle");
    if (water_index < 0 || water_index >= h->n_types)
        return fail(RSX_INVALID_ARG, "water_index outside the factor table");
    if (!std::isfinite(weight))
        return fail(RSX_INVALID_ARG, "water weight must be finite");
    if (weight != 0.f && !rsasa && h->rsasa.empty())
        return fail(RSX_INVALID_ARG, "a non-zero water weight needs rsasa");
    RSX_TRY_CUDA(cudaSetDevice(h->device), "cudaSetDevice");
    if (weight != 0.f && !h->d_rsasa) {
        const size_t M = (size_t)std::max(h->n_members, 1);
        RSX_TRY(dev_alloc((void **)&h->d_rsasa, sizeof(float) * std::max(h->n_total, 1),
                          "rsasa"));
        RSX_TRY(dev_alloc((void **)&h->d_water_sums,
                          sizeof(double) * (M * h->n_types + 2 * M), "rsasa sums"));
    }
    if (rsasa) {
        for (int i = 0; i < h->n_total; ++i)
            if (!std::isfinite(rsasa[i]))
                return fail(RSX_INVALID_ARG, "rsasa must be finite");
        h->rsasa.assign(rsasa, rsasa + h->n_total);
        h->water_dirty = true;
    }
    // weight and water column are arguments of the captured kernels
    // (a tile shape tuned without water runs capped at 128 q and two pairs)
    if (weight != h->water_weight || water_index != h->water_index)
        drop_graphs(h);
    h->water_weight = weight;
    h->water_index = water_index;
    return ok();
}

rsx_status rsx_batch_timing(rsx_batch *h, float *ms_last_pass)
{
    if (!h)
        return fail(RSX_ALG_NOT_INITIALIZED, "null rsx_batch handle");
    if (ms_last_pass)
        *ms_last_pass = h->last_ms;
    return ok();
}

rsx_status rsx_batch_config(rsx_batch *h, int *q_slab, int *n_items, int *persistent_ctas,
                            int *uniform_q)
{
    if (!h)
        return fail(RSX_ALG_NOT_INITIALIZED, "null rsx_batch handle");
    if (q_slab)
        *q_slab = h->q_slab;
    if (n_items)
        *n_items = (int)h->items.size();
    if (persistent_ctas)
        *persistent_ctas = h->fwd_grid;
    if (uniform_q)
        *uniform_q = h->uniform ? 1 : 0;
    return ok();
}

} // extern "C"
