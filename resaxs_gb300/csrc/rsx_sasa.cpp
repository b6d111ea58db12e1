// Dot-sphere SASA handle behind the C ABI: replaces rsasa_cl_gpu<float,float>
// (resaxslib/src/rsasa_cl_gpu_alg.cpp) -- host cell list, one H2D copy per
// call, counts back.  Dot sets are generated here from the reference's
// formulas (resaxslib/src/rsasa_algorithm.cpp).
#include "rsx_host.h"
#include "rsx_sasa_internal.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

using namespace rsx;

struct rsx_sasa {
    int device = -1;
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int n = 0, n_dots = 0;
    float probe = 0.f;
    std::vector<float> unit;
    float *d_unit = nullptr;
    unsigned char *d_buf = nullptr, *h_buf = nullptr;
    size_t buf_cap = 0;
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
    dev_free(h->d_unit);
    dev_free(h->d_buf);
    dev_free(h->d_counts);
    dev_free(h->d_tests);
    host_free_pinned(h->h_buf);
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

// Cell list of the atoms on the host, packed into the pinned buffer:
// atoms (float4 x,y,z,r) | cell coords (int3) | caller index | cell starts.
rsx_status pack_cells(rsx_sasa *h, const rsx_body *atoms, const float *radii, SasaArgs &a,
                      size_t &bytes_out)
{
    const int n = h->n;
    float lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0}, rmax = 0.f;
    for (int i = 0; i < n; ++i) {
        const float p[3] = {atoms[i].x, atoms[i].y, atoms[i].z};
        if (!std::isfinite(p[0]) || !std::isfinite(p[1]) || !std::isfinite(p[2]))
            return fail(RSX_INVALID_ARG, "atom " + std::to_string(i) + " has a non-finite position");
        if (!(radii[i] >= 0.f) || !std::isfinite(radii[i]))
            return fail(RSX_INVALID_ARG, "atom " + std::to_string(i) + " has an invalid radius");
        for (int c = 0; c < 3; ++c) {
            if (i == 0 || p[c] < lo[c])
                lo[c] = p[c];
            if (i == 0 || p[c] > hi[c])
                hi[c] = p[c];
        }
        rmax = std::max(rmax, radii[i]);
    }
    // a dot of atom i can only be occluded by an atom within r_i + r_b + 2P
    double cell = 2.0 * rmax + 2.0 * h->probe + 0.02;
    int dims[3];
    for (;;) {
        double total = 1.0;
        for (int c = 0; c < 3; ++c) {
            dims[c] = (int)std::floor((hi[c] - lo[c]) / cell) + 1;
            total *= dims[c];
        }
        if (total <= 4.0 * n + 4096.0)
            break;
        cell *= 1.5; // sparse, wide boxes: fewer, larger cells (still exact)
    }
    const int n_cells = dims[0] * dims[1] * dims[2];
    const size_t off_cell = sizeof(float4) * (size_t)n;
    const size_t off_orig = off_cell + sizeof(int) * 3 * (size_t)n;
    const size_t off_start = off_orig + sizeof(int) * (size_t)n;
    const size_t bytes = off_start + sizeof(int) * (size_t)(n_cells + 1);
    if (bytes > h->buf_cap) {
        dev_free(h->d_buf);
        host_free_pinned(h->h_buf);
        h->d_buf = h->h_buf = nullptr;
        h->buf_cap = 0;
        const size_t cap = bytes + bytes / 4 + 4096;
        RSX_TRY(dev_alloc((void **)&h->d_buf, cap, "sasa cells"));
        RSX_TRY(host_alloc_pinned((void **)&h->h_buf, cap, "sasa staging"));
        h->buf_cap = cap;
    }
    // the staging buffer may still feed the previous call's copy
    RSX_TRY_CUDA(cudaStreamSynchronize(h->st), "sasa staging");
    std::vector<int> cid(n), ccoord(3 * (size_t)n);
    int *start = reinterpret_cast<int *>(h->h_buf + off_start);
    std::memset(start, 0, sizeof(int) * (n_cells + 1));
    for (int i = 0; i < n; ++i) {
        const float p[3] = {atoms[i].x, atoms[i].y, atoms[i].z};
        int c3[3];
        for (int c = 0; c < 3; ++c) {
            int v = (int)std::floor((p[c] - lo[c]) / cell);
            c3[c] = std::min(std::max(v, 0), dims[c] - 1);
            ccoord[3 * (size_t)i + c] = c3[c];
        }
        cid[i] = (c3[0] * dims[1] + c3[1]) * dims[2] + c3[2];
        start[cid[i] + 1]++;
    }
    for (int c = 0; c < n_cells; ++c)
        start[c + 1] += start[c];
    std::vector<int> fill(start, start + n_cells);
    float4 *pa = reinterpret_cast<float4 *>(h->h_buf);
    int *pc = reinterpret_cast<int *>(h->h_buf + off_cell);
    int *po = reinterpret_cast<int *>(h->h_buf + off_orig);
    for (int i = 0; i < n; ++i) {
        const int s = fill[cid[i]]++;
        pa[s] = make_float4(atoms[i].x, atoms[i].y, atoms[i].z, radii[i]);
        pc[3 * s + 0] = ccoord[3 * (size_t)i + 0];
        pc[3 * s + 1] = ccoord[3 * (size_t)i + 1];
        pc[3 * s + 2] = ccoord[3 * (size_t)i + 2];
        po[s] = i;
    }
    a.atoms = reinterpret_cast<const float4 *>(h->d_buf);
    a.cell_of = reinterpret_cast<const int *>(h->d_buf + off_cell);
    a.orig_index = reinterpret_cast<const int *>(h->d_buf + off_orig);
    a.cell_start = reinterpret_cast<const int *>(h->d_buf + off_start);
    a.dims[0] = dims[0];
    a.dims[1] = dims[1];
    a.dims[2] = dims[2];
    a.max_radius = rmax;
    bytes_out = bytes;
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

rsx_status rsx_sasa_create(int n_atoms, const float *unit_dots, int n_dots, float probe,
                           int device, rsx_sasa **out)
{
    if (!out)
        return fail(RSX_INVALID_ARG, "out handle pointer is null");
    *out = nullptr;
    if (n_atoms < 0 || !unit_dots || n_dots <= 0 || n_dots > 4096 || !(probe >= 0.f) ||
        !std::isfinite(probe))
        return fail(RSX_INVALID_ARG, "need n_atoms >= 0, 1..4096 unit dots and probe >= 0");
    int dev = -1;
    RSX_TRY(select_device(device, &dev));
    DeviceGuard g(dev);
    cudaSetDevice(dev);
    rsx_sasa *h = new rsx_sasa();
    h->device = dev;
    h->n = n_atoms;
    h->n_dots = n_dots;
    h->probe = probe;
    h->unit.assign(unit_dots, unit_dots + 3 * (size_t)n_dots);
    auto bail = [&](rsx_status s) {
        sasa_release(h);
        return s;
    };
    cudaError_t e = cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking);
    if (e == cudaSuccess)
        e = cudaEventCreate(&h->e0);
    if (e == cudaSuccess)
        e = cudaEventCreate(&h->e1);
    if (e != cudaSuccess)
        return bail(cuda_status(e, "sasa stream/events"));
    rsx_status s;
    if ((s = dev_alloc((void **)&h->d_unit, sizeof(float) * 3 * n_dots, "unit dots")) != RSX_OK)
        return bail(s);
    if ((s = dev_alloc((void **)&h->d_counts, sizeof(unsigned) * std::max(n_atoms, 1), "counts")) !=
        RSX_OK)
        return bail(s);
    if ((s = dev_alloc((void **)&h->d_tests, sizeof(unsigned long long), "tests")) != RSX_OK)
        return bail(s);
    if ((s = host_alloc_pinned((void **)&h->h_counts, sizeof(unsigned) * std::max(n_atoms, 1),
                               "pinned counts")) != RSX_OK)
        return bail(s);
    if ((s = host_alloc_pinned((void **)&h->h_tests, sizeof(unsigned long long), "pinned tests")) !=
        RSX_OK)
        return bail(s);
    e = cudaMemcpyAsync(h->d_unit, h->unit.data(), sizeof(float) * 3 * n_dots,
                        cudaMemcpyHostToDevice, h->st);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(h->st);
    if (e != cudaSuccess)
        return bail(cuda_status(e, "upload dots"));
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
    if ((!atoms || !radii) && h->n > 0)
        return fail(RSX_INVALID_ARG, "atoms / radii are null");
    if (!out_counts)
        return fail(RSX_INVALID_ARG, "counts output is null");
    RSX_TRY_CUDA(cudaSetDevice(h->device), "cudaSetDevice");
    if (h->n == 0)
        return ok();
    SasaArgs a{};
    size_t bytes = 0;
    RSX_TRY(pack_cells(h, atoms, radii, a, bytes));
    a.unit = h->d_unit;
    a.counts = h->d_counts;
    a.tests = h->d_tests;
    a.n_atoms = h->n;
    a.n_dots = h->n_dots;
    a.probe = h->probe;
    RSX_TRY_CUDA(cudaMemcpyAsync(h->d_buf, h->h_buf, bytes, cudaMemcpyHostToDevice, h->st),
                 "upload cells");
    RSX_TRY_CUDA(cudaMemsetAsync(h->d_tests, 0, sizeof(unsigned long long), h->st), "zero tests");
    RSX_TRY_CUDA(cudaEventRecord(h->e0, h->st), "event");
    RSX_LAUNCH(launch_sasa(a, h->st), "sasa kernel");
    RSX_TRY_CUDA(cudaEventRecord(h->e1, h->st), "event");
    RSX_TRY_CUDA(cudaMemcpyAsync(h->h_counts, h->d_counts, sizeof(unsigned) * h->n,
                                 cudaMemcpyDeviceToHost, h->st),
                 "read counts");
    RSX_TRY_CUDA(cudaMemcpyAsync(h->h_tests, h->d_tests, sizeof(unsigned long long),
                                 cudaMemcpyDeviceToHost, h->st),
                 "read tests");
    RSX_TRY_CUDA(cudaStreamSynchronize(h->st), "sasa");
    cudaEventElapsedTime(&h->last_ms, h->e0, h->e1);
    h->last_tests = *h->h_tests;
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
