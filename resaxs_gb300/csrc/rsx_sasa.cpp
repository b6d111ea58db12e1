// Dot-sphere SASA handle behind the C ABI: replaces rsasa_cl_gpu<float,float>
// (resaxslib/src/rsasa_cl_gpu_alg.cpp) and rsasa_cpu_alg<float,float>
// (resaxslib/src/rsasa_cpu_alg.cpp).  Two forms:
//  * unit: one set of unit directions, dot = unit * (r_i + P), radii per atom;
//  * typed: the reference's own layout, pre-scaled dots per atom type with
//    padding (dots_map_[type * stride + dot], rsasa_cl_gpu_alg.cpp:59-89) and
//    radii per type.
// Per call: one pass over the atoms on the host (checks, bounding box), one
// H2D copy, the cell list and the occlusion pass on the GPU, counts back.
// Dot sets are generated here from the reference's formulas
// (resaxslib/src/rsasa_algorithm.cpp).
#include "rsx_host.h"
#include "rsx_sasa_internal.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <numeric>
#include <vector>

using namespace rsx;

struct rsx_sasa {
    int device = -1;
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int n = 0;
    bool typed = false;
    int n_types = 1, n_dots = 0; // n_dots: unit form
    float probe = 0.f;
    float unit_reach = 0.f;
    std::vector<float> type_radius, dot_reach;
    std::vector<int> dots_of_type; // accessible-dot denominator per type (typed form)
    float4 *d_dots = nullptr;
    int *d_group_base = nullptr, *d_group_count = nullptr;
    float *d_dot_reach = nullptr, *d_type_radius = nullptr;
    // per-call buffers
    unsigned char *d_in = nullptr, *h_in = nullptr; // atoms float4 [n] | radii [n]
    float4 *d_atoms = nullptr;
    int *d_cell_of = nullptr, *d_rank_of = nullptr, *d_orig = nullptr, *d_type_of = nullptr;
    int *d_cell_sorted = nullptr;
    int *d_cell_count = nullptr, *d_cell_start = nullptr; // [4 n + 4097] each
    int cells_cap = 0;
    SasaGeom *d_geom = nullptr, *h_geom = nullptr;
    unsigned *d_counts = nullptr, *h_counts = nullptr;
    unsigned long long *d_tests = nullptr, *h_tests = nullptr;
    float last_ms = 0.f;
    unsigned long long last_tests = 0;
};

namespace {

rsx_status sasa_release(rsx_sasa *h)
{
    if (!h)
        return RSX_OK;
    DeviceGuard g(h->device);
    if (h->st)
        cudaStreamSynchronize(h->st);
    for (void *p : {(void *)h->d_dots, (void *)h->d_group_base, (void *)h->d_group_count,
                    (void *)h->d_dot_reach, (void *)h->d_type_radius, (void *)h->d_in,
                    (void *)h->d_atoms, (void *)h->d_cell_of, (void *)h->d_rank_of,
                    (void *)h->d_orig, (void *)h->d_type_of, (void *)h->d_cell_sorted,
                    (void *)h->d_cell_count, (void *)h->d_cell_start, (void *)h->d_counts,
                    (void *)h->d_tests, (void *)h->d_geom})
        dev_free(p);
    host_free_pinned(h->h_in);
    host_free_pinned(h->h_geom);
    host_free_pinned(h->h_counts);
    host_free_pinned(h->h_tests);
    if (h->e0)
        cudaEventDestroy(h->e0);
    if (h->e1)
        cudaEventDestroy(h->e1);
    if (h->st)
        cudaStreamDestroy(h->st);
    delete h;
    return RSX_OK;
}

// Orders idx[b, e) so that every run of 32 dots is compact on the sphere:
// halves along the axis of largest extent, cut at a multiple of 32.  The
// counts do not depend on the order; the lanes of a warp then tend to meet
// their first occluder together.
void compact_groups(const std::vector<float4> &d, std::vector<int> &idx, int b, int e)
{
    const int n = e - b;
    if (n <= 32)
        return;
    float lo[3] = {3.4e38f, 3.4e38f, 3.4e38f}, hi[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
    for (int k = b; k < e; ++k) {
        const float v[3] = {d[idx[k]].x, d[idx[k]].y, d[idx[k]].z};
        for (int a = 0; a < 3; ++a) {
            lo[a] = std::min(lo[a], v[a]);
            hi[a] = std::max(hi[a], v[a]);
        }
    }
    int ax = 0;
    for (int a = 1; a < 3; ++a)
        if (hi[a] - lo[a] > hi[ax] - lo[ax])
            ax = a;
    const int groups = (n + 31) / 32;
    const int cut = b + 32 * ((groups + 1) / 2);
    auto key = [&](int k) { return ax == 0 ? d[k].x : (ax == 1 ? d[k].y : d[k].z); };
    std::nth_element(idx.begin() + b, idx.begin() + cut, idx.begin() + e,
                     [&](int p, int q) { return key(p) < key(q) || (key(p) == key(q) && p < q); });
    compact_groups(d, idx, b, cut);
    compact_groups(d, idx, cut, e);
}

// Appends one dot set as 32-dot groups (x not finite: padding) to `table`;
// returns the number of groups and the largest |d| of its fully finite dots.
int append_groups(const std::vector<float4> &set, std::vector<float4> &table, float *reach)
{
    std::vector<int> idx(set.size());
    std::iota(idx.begin(), idx.end(), 0);
    // dots with a non-finite y or z can never be occluded: they go last
    auto finite3 = [&](int k) {
        return std::isfinite(set[k].y) && std::isfinite(set[k].z);
    };
    const auto mid = std::stable_partition(idx.begin(), idx.end(), finite3);
    compact_groups(set, idx, 0, (int)(mid - idx.begin()));
    double r = 0.0;
    for (auto it = idx.begin(); it != mid; ++it) {
        const float4 &v = set[*it];
        r = std::max(r, std::sqrt((double)v.x * v.x + (double)v.y * v.y + (double)v.z * v.z));
    }
    *reach = (float)(r * (1.0 + 1e-6));
    const int groups = ((int)set.size() + 31) / 32;
    const float nan = std::nanf("");
    for (int k = 0; k < groups * 32; ++k)
        table.push_back(k < (int)set.size() ? set[idx[k]] : make_float4(nan, 0.f, 0.f, 0.f));
    return groups;
}

rsx_status upload_dots(rsx_sasa *h, const std::vector<float4> &table,
                       const std::vector<int> &base, const std::vector<int> &count)
{
    RSX_TRY(dev_alloc((void **)&h->d_dots, sizeof(float4) * std::max<size_t>(table.size(), 1),
                      "sasa dots"));
    RSX_TRY(dev_alloc((void **)&h->d_group_base, sizeof(int) * base.size(), "sasa groups"));
    RSX_TRY(dev_alloc((void **)&h->d_group_count, sizeof(int) * count.size(), "sasa groups"));
    RSX_TRY(dev_alloc((void **)&h->d_dot_reach, sizeof(float) * h->dot_reach.size(), "sasa reach"));
    RSX_TRY(dev_alloc((void **)&h->d_type_radius, sizeof(float) * h->type_radius.size(),
                      "sasa radii"));
    const cudaMemcpyKind k = cudaMemcpyHostToDevice;
    cudaError_t e = cudaMemcpyAsync(h->d_dots, table.data(), sizeof(float4) * table.size(), k, h->st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(h->d_group_base, base.data(), sizeof(int) * base.size(), k, h->st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(h->d_group_count, count.data(), sizeof(int) * count.size(), k, h->st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(h->d_dot_reach, h->dot_reach.data(), sizeof(float) * h->dot_reach.size(),
                            k, h->st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(h->d_type_radius, h->type_radius.data(),
                            sizeof(float) * h->type_radius.size(), k, h->st);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(h->st); // the host vectors are temporaries
    return cuda_status(e, "upload dots");
}

rsx_status new_handle(int n_atoms, float probe, int device, rsx_sasa **out)
{
    int dev = -1;
    RSX_TRY(select_device(device, &dev));
    DeviceGuard g(dev);
    RSX_TRY_CUDA(cudaSetDevice(dev), "cudaSetDevice");
    rsx_sasa *h = new rsx_sasa();
    h->device = dev;
    h->n = n_atoms;
    h->probe = probe;
    cudaError_t e = cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking);
    if (e == cudaSuccess)
        e = cudaEventCreate(&h->e0);
    if (e == cudaSuccess)
        e = cudaEventCreate(&h->e1);
    rsx_status s = cuda_status(e, "sasa stream/events");
    const size_t n1 = (size_t)std::max(n_atoms, 1);
    if (s == RSX_OK)
        s = dev_alloc((void **)&h->d_in, (sizeof(float4) + sizeof(float)) * n1, "sasa atoms");
    if (s == RSX_OK)
        s = host_alloc_pinned((void **)&h->h_in, (sizeof(float4) + sizeof(float)) * n1,
                              "sasa staging");
    if (s == RSX_OK)
        s = dev_alloc((void **)&h->d_atoms, sizeof(float4) * n1, "sasa cell atoms");
    for (int **p : {&h->d_cell_of, &h->d_rank_of, &h->d_orig, &h->d_type_of, &h->d_cell_sorted})
        if (s == RSX_OK)
            s = dev_alloc((void **)p, sizeof(int) * n1, "sasa cell index");
    if (s == RSX_OK)
        s = dev_alloc((void **)&h->d_counts, sizeof(unsigned) * n1, "counts");
    if (s == RSX_OK)
        s = dev_alloc((void **)&h->d_tests, sizeof(unsigned long long), "tests");
    if (s == RSX_OK)
        s = host_alloc_pinned((void **)&h->h_counts, sizeof(unsigned) * n1, "pinned counts");
    if (s == RSX_OK)
        s = host_alloc_pinned((void **)&h->h_tests, sizeof(unsigned long long), "pinned tests");
    // the cell grid has at most 4 n + 4096 cells (sasa_plan_kernel)
    h->cells_cap = 4 * (int)n1 + 4097;
    if (s == RSX_OK)
        s = dev_alloc((void **)&h->d_cell_count, sizeof(int) * (size_t)h->cells_cap, "sasa cells");
    if (s == RSX_OK)
        s = dev_alloc((void **)&h->d_cell_start, sizeof(int) * (size_t)h->cells_cap, "sasa cells");
    if (s == RSX_OK)
        s = dev_alloc((void **)&h->d_geom, sizeof(SasaGeom), "sasa geometry");
    if (s == RSX_OK)
        s = host_alloc_pinned((void **)&h->h_geom, sizeof(SasaGeom), "pinned sasa geometry");
    if (s != RSX_OK) {
        sasa_release(h);
        return s;
    }
    *out = h;
    return RSX_OK;
}

// Checks the atoms, stages them, builds the cell list and runs the occlusion
// pass; counts land in h->h_counts.
rsx_status run(rsx_sasa *h, const rsx_body *atoms, const float *radii)
{
    const int n = h->n;
    // the staging buffer may still feed the previous call's copy
    RSX_TRY_CUDA(cudaStreamSynchronize(h->st), "sasa staging");
    std::memcpy(h->h_in, atoms, sizeof(float4) * (size_t)n);
    size_t bytes = sizeof(float4) * (size_t)n;
    if (!h->typed) {
        std::memcpy(h->h_in + bytes, radii, sizeof(float) * (size_t)n);
        bytes += sizeof(float) * (size_t)n;
    }
    // The checks, the bounding box and the cell grid are formed on the GPU
    // (sasa_geom_kernel, sasa_plan_kernel); the host reads the verdict with
    // the counts and names the first bad atom only when there is one.
    SasaCellArgs c{};
    c.atoms_in = reinterpret_cast<const float4 *>(h->d_in);
    c.radii_in = h->typed ? nullptr : reinterpret_cast<const float *>(h->d_in + sizeof(float4) * n);
    c.type_radius = h->d_type_radius;
    c.cell_count = h->d_cell_count;
    c.cell_start = h->d_cell_start;
    c.cell_of = h->d_cell_of;
    c.rank_of = h->d_rank_of;
    c.atoms = h->d_atoms;
    c.orig_index = h->d_orig;
    c.type_of = h->d_type_of;
    c.cell_sorted = h->d_cell_sorted;
    c.geom = h->d_geom;
    c.dot_reach = h->d_dot_reach;
    c.unit_reach = h->unit_reach;
    c.probe = h->probe;
    c.n_atoms = n;
    c.n_types = h->typed ? h->n_types : 1;
    c.cells_cap = h->cells_cap;
    SasaArgs a{};
    a.atoms = h->d_atoms;
    a.orig_index = h->d_orig;
    a.type_of = h->typed ? h->d_type_of : nullptr;
    a.cell_id = h->d_cell_sorted;
    a.cell_start = h->d_cell_start;
    a.dots = h->d_dots;
    a.group_base = h->d_group_base;
    a.group_count = h->d_group_count;
    a.dot_reach = h->d_dot_reach;
    a.unit_reach = h->unit_reach;
    a.typed = h->typed ? 1 : 0;
    a.counts = h->d_counts;
    a.tests = h->d_tests;
    a.geom = h->d_geom;
    a.n_atoms = n;
    a.probe = h->probe;
    RSX_TRY_CUDA(cudaMemcpyAsync(h->d_in, h->h_in, bytes, cudaMemcpyHostToDevice, h->st),
                 "upload atoms");
    RSX_TRY_CUDA(cudaMemsetAsync(h->d_tests, 0, sizeof(unsigned long long), h->st), "zero tests");
    RSX_TRY_CUDA(cudaEventRecord(h->e0, h->st), "event");
    RSX_LAUNCH(launch_sasa_cells(c, h->st), "sasa cell list");
    RSX_LAUNCH(launch_sasa(a, h->st), "sasa kernel");
    RSX_TRY_CUDA(cudaEventRecord(h->e1, h->st), "event");
    RSX_TRY_CUDA(cudaMemcpyAsync(h->h_counts, h->d_counts, sizeof(unsigned) * n,
                                 cudaMemcpyDeviceToHost, h->st),
                 "read counts");
    RSX_TRY_CUDA(cudaMemcpyAsync(h->h_tests, h->d_tests, sizeof(unsigned long long),
                                 cudaMemcpyDeviceToHost, h->st),
                 "read tests");
    RSX_TRY_CUDA(cudaMemcpyAsync(h->h_geom, h->d_geom, sizeof(SasaGeom), cudaMemcpyDeviceToHost,
                                 h->st),
                 "read sasa geometry");
    RSX_TRY_CUDA(cudaStreamSynchronize(h->st), "sasa");
    if (h->h_geom->bad) {
        for (int i = 0; i < n; ++i) {
            if (!std::isfinite(atoms[i].x) || !std::isfinite(atoms[i].y) ||
                !std::isfinite(atoms[i].z))
                return fail(RSX_INVALID_ARG, "atom " + std::to_string(i) + " has a non-finite position");
            unsigned t;
            std::memcpy(&t, &atoms[i].w, 4);
            if (h->typed && t >= (unsigned)h->n_types)
                return fail(RSX_INVALID_ARG, "atom " + std::to_string(i) + " has type " +
                                                 std::to_string(t) + " outside the dot map");
            if (!h->typed && (!(radii[i] >= 0.f) || !std::isfinite(radii[i])))
                return fail(RSX_INVALID_ARG, "atom " + std::to_string(i) + " has an invalid radius");
        }
        return fail(RSX_INVALID_ARG, "invalid atoms");
    }
    cudaEventElapsedTime(&h->last_ms, h->e0, h->e1);
    h->last_tests = *h->h_tests;
    return RSX_OK;
}

} // namespace

extern "C" {

rsx_status rsx_sasa_fibonacci_dots(int n_dots, float *out_xyz)
{
    // rsasa_algorithm.cpp:96-116 with n = n_dots / 2, in FP32 as there
    if (!out_xyz || n_dots < 2 || (n_dots & 1))
        return fail(RSX_INVALID_ARG, "n_dots must be even and >= 2");
    const int n = n_dots / 2;
    const float phi = (1.0f + std::sqrt(5.0f)) / 2.0f;
    const float pi_f = (float)3.14159265358979323846;
    int k = 0;
    for (int i = -(n - 1); i <= n; ++i, ++k) {
        const float theta = 2 * pi_f * (float)i / phi;
        const float sphi = (float)i / (float)n;
        const float cphi = (float)(std::sqrt((double)((n + i) * (n - i))) / n);
        out_xyz[3 * k + 0] = cphi * std::sin(theta);
        out_xyz[3 * k + 1] = cphi * std::cos(theta);
        out_xyz[3 * k + 2] = sphi;
    }
    return ok();
}

rsx_status rsx_sasa_dodeca_icosa_dots(float *out_xyz)
{
    // the 32 unit directions of create_dodeca_icosa_dots
    // (rsasa_algorithm.cpp:156-208): 20 dodecahedron vertices and 12
    // icosahedron vertices, ext_radius = 1
    if (!out_xyz)
        return fail(RSX_INVALID_ARG, "output is null");
    const float phi = (1.0f + std::sqrt(5.0f)) / 2.0f;
    const float v1 = 1 / std::sqrt(3.0f);
    const float v2 = (1 / phi) * v1, v3 = phi * v1;
    const double pi = 3.14159265358979323846;
    const float ico = (float)((std::sqrt(5.0) + 5) / 10 /
                              std::sqrt(3 - 1 / std::pow(phi * std::cos(3 * pi / 10), 2)));
    const float P = phi * ico;
    const float d[32][3] = {
        {v1, v1, v1},   {v1, v1, -v1},  {v1, -v1, v1},  {v1, -v1, -v1}, {-v1, v1, v1},
        {-v1, v1, -v1}, {-v1, -v1, v1}, {-v1, -v1, -v1}, {0, v2, v3},    {0, v2, -v3},
        {0, -v2, v3},   {0, -v2, -v3},  {v2, v3, 0},    {v2, -v3, 0},   {-v2, v3, 0},
        {-v2, -v3, 0},  {v3, 0, v2},    {v3, 0, -v2},   {-v3, 0, v2},   {-v3, 0, -v2},
        {ico, 0, P},    {ico, 0, -P},   {-ico, 0, P},   {-ico, 0, -P},  {0, P, ico},
        {0, P, -ico},   {0, -P, ico},   {0, -P, -ico},  {P, ico, 0},    {P, -ico, 0},
        {-P, ico, 0},   {-P, -ico, 0}};
    std::memcpy(out_xyz, d, sizeof d);
    return ok();
}

rsx_status rsx_sasa_sphere_dots(int kind, float radius, float dot_density, float probe,
                                float *out_xyzw, int cap, int *n_out)
{
    // dot_spheres_params::create_* (rsasa_algorithm.cpp:60-208) in FLT_T =
    // float, operation for operation: the dots are pre-scaled by
    // ext = radius + probe and carry the radius in w.
    if (!n_out || (!out_xyzw && cap > 0) || cap < 0)
        return fail(RSX_INVALID_ARG, "null output");
    *n_out = 0;
    if (!std::isfinite(radius) || !std::isfinite(probe) || !std::isfinite(dot_density))
        return fail(RSX_INVALID_ARG, "radius, probe and density must be finite");
    const float pi_f = (float)3.14159265358979323846;
    const float ext = radius + probe;
    std::vector<float4> d;
    auto sphere = [&](float n_sect) { // create_sphere_dots (:38-58)
        const float n_vert_sect = 0.5f * n_sect;
        for (unsigned i = 0; (float)i < n_vert_sect; i++) {
            const float phi = (pi_f * (float)i) / n_vert_sect;
            const float z = std::cos(phi) * ext;
            const float xy = std::sin(phi);
            const float horz_count = xy * n_sect;
            for (unsigned j = 0; (float)j < horz_count - 1; j++) {
                const float theta = (2 * pi_f * (float)j) / horz_count;
                const float x = xy * std::cos(theta) * ext;
                const float y = xy * std::sin(theta) * ext;
                d.push_back(make_float4(x, y, z, radius));
                if (d.size() > (size_t)1 << 20)
                    return false;
            }
        }
        return true;
    };
    const float phi = (1.0f + std::sqrt(5.0f)) / 2.0f;
    switch (kind) {
    case RSX_DOTS_LATITUDE: {
        // create_dots (:60-65): n_sect = 2 pi r sqrt(density)
        if (!(dot_density >= 0.f))
            return fail(RSX_INVALID_ARG, "dot density must be >= 0");
        const float n_sect = 2 * pi_f * radius * std::sqrt(dot_density);
        if (!sphere(n_sect))
            return fail(RSX_INVALID_ARG, "more than 2^20 dots");
        break;
    }
    case RSX_DOTS_32:
        sphere(10.5f); // create_32_dots (:67-71)
        break;
    case RSX_DOTS_FIBONACCI: { // create_fibonacci_dots (:96-116)
        const int n = 32;
        for (int i = -(n - 1); i <= n; ++i) {
            const float theta = 2 * pi_f * i / phi;
            const float sphi = static_cast<float>(i) / n;
            const float cphi = static_cast<float>(std::sqrt((double)((n + i) * (n - i))) / n);
            d.push_back(make_float4(cphi * std::sin(theta) * ext, cphi * std::cos(theta) * ext,
                                    sphi * ext, radius));
        }
        break;
    }
    case RSX_DOTS_DODECAHEDRON:
    case RSX_DOTS_DODECA_ICOSA: { // (:118-154), (:156-208)
        const float r_phi = 1 / phi;
        const float r_sqrt3 = 1 / std::sqrt(3.0f);
        const float v1 = r_sqrt3 * ext, v2 = r_phi * v1, v3 = phi * v1;
        const float dod[20][3] = {
            {v1, v1, v1},  {v1, v1, -v1},  {v1, -v1, v1},  {v1, -v1, -v1}, {-v1, v1, v1},
            {-v1, v1, -v1}, {-v1, -v1, v1}, {-v1, -v1, -v1}, {0, v2, v3},   {0, v2, -v3},
            {0, -v2, v3},  {0, -v2, -v3},  {v2, v3, 0},    {v2, -v3, 0},   {-v2, v3, 0},
            {-v2, -v3, 0}, {v3, 0, v2},    {v3, 0, -v2},   {-v3, 0, v2},   {-v3, 0, -v2}};
        for (const auto &v : dod)
            d.push_back(make_float4(v[0], v[1], v[2], radius));
        if (kind == RSX_DOTS_DODECA_ICOSA) {
            const double pi = 3.14159265358979323846;
            const float ico = (float)((std::sqrt(5.0f) + 5) / 10 /
                                      std::sqrt(3 - 1 / std::pow(phi * std::cos(3 * pi / 10), 2)) *
                                      ext);
            const float pi_c = phi * ico;
            const float ic[12][3] = {{ico, 0, pi_c},  {ico, 0, -pi_c}, {-ico, 0, pi_c},
                                     {-ico, 0, -pi_c}, {0, pi_c, ico},  {0, pi_c, -ico},
                                     {0, -pi_c, ico}, {0, -pi_c, -ico}, {pi_c, ico, 0},
                                     {pi_c, -ico, 0}, {-pi_c, ico, 0}, {-pi_c, -ico, 0}};
            for (const auto &v : ic)
                d.push_back(make_float4(v[0], v[1], v[2], radius));
        }
        break;
    }
    default:
        return fail(RSX_INVALID_ARG, "unknown dot set kind");
    }
    *n_out = (int)d.size();
    if ((int)d.size() > cap)
        return fail(RSX_INVALID_ARG, "output holds " + std::to_string(cap) + " dots, the set has " +
                                         std::to_string(d.size()));
    if (!d.empty())
        std::memcpy(out_xyzw, d.data(), sizeof(float4) * d.size());
    return ok();
}

rsx_status rsx_sasa_create(int n_atoms, const float *unit_dots, int n_dots, float probe,
                           int device, rsx_sasa **out)
{
    if (!out)
        return fail(RSX_INVALID_ARG, "out handle pointer is null");
    *out = nullptr;
    if (n_atoms < 0 || n_atoms > kSasaMaxAtoms || !unit_dots || n_dots <= 0 ||
        n_dots > 32 * kSasaMaxGroups || !(probe >= 0.f) || !std::isfinite(probe))
        return fail(RSX_INVALID_ARG,
                    "need 0 <= n_atoms <= 2^28, 1..4096 unit dots and probe >= 0");
    std::vector<float4> set((size_t)n_dots);
    for (int k = 0; k < n_dots; ++k) {
        set[k] = make_float4(unit_dots[3 * k], unit_dots[3 * k + 1], unit_dots[3 * k + 2], 0.f);
        if (!std::isfinite(set[k].x) || !std::isfinite(set[k].y) || !std::isfinite(set[k].z))
            return fail(RSX_INVALID_ARG, "unit dot " + std::to_string(k) + " is not finite");
    }
    rsx_sasa *h = nullptr;
    RSX_TRY(new_handle(n_atoms, probe, device, &h));
    DeviceGuard g(h->device);
    h->n_dots = n_dots;
    std::vector<float4> table;
    float reach = 0.f;
    const int groups = append_groups(set, table, &reach);
    h->unit_reach = reach;
    h->dot_reach.assign(1, reach);
    h->type_radius.assign(1, 0.f);
    rsx_status s = upload_dots(h, table, {0}, {groups});
    if (s != RSX_OK) {
        sasa_release(h);
        return s;
    }
    *out = h;
    return ok();
}

rsx_status rsx_sasa_create_typed(int n_atoms, const float *dot_map, int n_types, int stride,
                                 const float *type_radii, float probe, int device,
                                 rsx_sasa **out)
{
    if (!out)
        return fail(RSX_INVALID_ARG, "out handle pointer is null");
    *out = nullptr;
    if (n_atoms < 0 || n_atoms > kSasaMaxAtoms || !dot_map || !type_radii || n_types <= 0 ||
        n_types > kSasaMaxTypes || stride <= 0 || stride > 32 * kSasaMaxGroups ||
        !(probe >= 0.f) || !std::isfinite(probe))
        return fail(RSX_INVALID_ARG, "need 0 <= n_atoms <= 2^28, 1..256 types, 1..4096 dots per "
                                     "type and probe >= 0");
    for (int t = 0; t < n_types; ++t)
        if (!(type_radii[t] >= 0.f) || !std::isfinite(type_radii[t]))
            return fail(RSX_INVALID_ARG, "type " + std::to_string(t) + " has an invalid radius");
    rsx_sasa *h = nullptr;
    RSX_TRY(new_handle(n_atoms, probe, device, &h));
    DeviceGuard g(h->device);
    h->typed = true;
    h->n_types = n_types;
    h->type_radius.assign(type_radii, type_radii + n_types);
    h->dot_reach.assign(n_types, 0.f);
    h->dots_of_type.assign(n_types, 0);
    std::vector<float4> table;
    std::vector<int> base(n_types), count(n_types);
    for (int t = 0; t < n_types; ++t) {
        // a dot whose x is not finite is padding (rsasa_cl_gpu_alg.cpp:72-86)
        std::vector<float4> set;
        for (int k = 0; k < stride; ++k) {
            const float *d = dot_map + 4 * ((size_t)t * stride + k);
            if (std::isfinite(d[0]))
                set.push_back(make_float4(d[0], d[1], d[2], 0.f));
        }
        h->dots_of_type[t] = (int)set.size();
        base[t] = (int)(table.size() / 32);
        count[t] = set.empty() ? 0 : append_groups(set, table, &h->dot_reach[t]);
    }
    rsx_status s = upload_dots(h, table, base, count);
    if (s != RSX_OK) {
        sasa_release(h);
        return s;
    }
    *out = h;
    return ok();
}

rsx_status rsx_sasa_destroy(rsx_sasa *h)
{
    sasa_release(h);
    return ok();
}

rsx_status rsx_sasa_counts(rsx_sasa *h, const rsx_body *atoms, const float *radii,
                           unsigned *out_counts)
{
    if (!h)
        return fail(RSX_ALG_NOT_INITIALIZED, "null rsx_sasa handle");
    if (h->typed)
        return fail(RSX_INVALID_ARG, "handle has a typed dot map: use rsx_sasa_counts_typed");
    if ((!atoms || !radii) && h->n > 0)
        return fail(RSX_INVALID_ARG, "atoms / radii are null");
    if (!out_counts)
        return fail(RSX_INVALID_ARG, "counts output is null");
    RSX_TRY_CUDA(cudaSetDevice(h->device), "cudaSetDevice");
    if (h->n == 0)
        return ok();
    RSX_TRY(run(h, atoms, radii));
    std::memcpy(out_counts, h->h_counts, sizeof(unsigned) * h->n);
    return ok();
}

rsx_status rsx_sasa_calc(rsx_sasa *h, const rsx_body *atoms, const float *radii, float *out_rsasa)
{
    if (!h)
        return fail(RSX_ALG_NOT_INITIALIZED, "null rsx_sasa handle");
    if (!out_rsasa)
        return fail(RSX_INVALID_ARG, "rsasa output is null");
    std::vector<unsigned> c(std::max(h->n, 1));
    RSX_TRY(rsx_sasa_counts(h, atoms, radii, c.data()));
    for (int i = 0; i < h->n; ++i) // rsasa_cl_gpu_alg.cpp:191-196
        out_rsasa[i] = static_cast<float>(c[i]) / h->n_dots;
    return ok();
}

rsx_status rsx_sasa_counts_typed(rsx_sasa *h, const rsx_body *atoms, unsigned *out_counts)
{
    if (!h)
        return fail(RSX_ALG_NOT_INITIALIZED, "null rsx_sasa handle");
    if (!h->typed)
        return fail(RSX_INVALID_ARG, "handle has unit dots: use rsx_sasa_counts");
    if (!atoms && h->n > 0)
        return fail(RSX_INVALID_ARG, "atoms are null");
    if (!out_counts)
        return fail(RSX_INVALID_ARG, "counts output is null");
    RSX_TRY_CUDA(cudaSetDevice(h->device), "cudaSetDevice");
    if (h->n == 0)
        return ok();
    RSX_TRY(run(h, atoms, nullptr));
    std::memcpy(out_counts, h->h_counts, sizeof(unsigned) * h->n);
    return ok();
}

rsx_status rsx_sasa_calc_typed(rsx_sasa *h, const rsx_body *atoms, float *out_rsasa)
{
    if (!h)
        return fail(RSX_ALG_NOT_INITIALIZED, "null rsx_sasa handle");
    if (!out_rsasa)
        return fail(RSX_INVALID_ARG, "rsasa output is null");
    std::vector<unsigned> c(std::max(h->n, 1));
    RSX_TRY(rsx_sasa_counts_typed(h, atoms, c.data()));
    for (int i = 0; i < h->n; ++i) { // rsasa_cl_gpu_alg.cpp:191-196: count / dots of the type
        unsigned t;
        std::memcpy(&t, &atoms[i].w, 4);
        out_rsasa[i] = static_cast<float>(c[i]) / h->dots_of_type[t];
    }
    return ok();
}

rsx_status rsx_sasa_stats(rsx_sasa *h, unsigned long long *tests, float *ms_kernel)
{
    if (!h)
        return fail(RSX_ALG_NOT_INITIALIZED, "null rsx_sasa handle");
    if (tests)
        *tests = h->last_tests;
    if (ms_kernel)
        *ms_kernel = h->last_ms;
    return ok();
}

} // extern "C"
