// Debye forward for callers that cannot allocate device memory.
//
// Some callers of this library run where device allocation is not available
// to them: inside a host framework that owns every device allocation through
// its own pool (and forbids cudaMalloc from plug-in code), or on a stream that
// is being driven by a scheduler which must not see allocator calls between
// its launches.  They already hold their inputs and outputs on the device and
// need the curve computed in place.  rsx_calc_saxs_curve_device_noalloc serves
// them: it takes device pointers only, and the working memory of the pair
// kernel (the FP64 per-item partial sums that rsx_debye_calc keeps in a
// cudaMalloc'ed buffer) lives in one file-scope static __device__ array,
// g_noalloc_scratch, of kNoAllocScratchBytes = 8 MiB.  Every GPU that loads
// librsx holds that array until the process exits.
//
// The kernel is a variant of the forward pair kernel of debye_kernels.cu that
// works on the caller's body order (no type sort, which would need working
// memory for the permuted copy): each J body carries its own form factor row,
// read from shared memory per pair, and each pair uses the direct range-
// reduced sine for every q (no uniform-grid recurrence, since the q vector
// stays on the device).  It is therefore several times slower than
// rsx_debye_calc and computes the same sum to the same 1e-5 tolerance.
#include "rsx_host.h"
#include "debye_device.cuh"

#include <mutex>

namespace rsx {

constexpr size_t kNoAllocScratchBytes = size_t(8) << 20;
constexpr size_t kNoAllocScratchDoubles = kNoAllocScratchBytes / sizeof(double);
// the first 32 doubles hold the error word; partial sums follow
constexpr size_t kNoAllocHeader = 32;
constexpr int kNoAllocQS = 16;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchDoubles];

struct NoAllocArgs {
    const float4 *bodies; // caller order, .w = type bits
    const float *q;       // [n_q]
    const float *ff;      // [n_q][n_types]
    float *out;           // [n_q]
    double *partial;      // [n_q][n_items] inside the static scratch
    unsigned *err;        // error word inside the static scratch
    int n, n_q, n_types, n_blocks, jchunk, n_items;
};

// item index -> (I-block, first J-block) for rows of ceil((nb - bi) / jchunk) items
__device__ __forceinline__ void decode_item(int item, int nb, int jc, int &bi, int &bj0)
{
    int b = 0;
    for (; b < nb; ++b) {
        const int cnt = (nb - b + jc - 1) / jc;
        if (item < cnt)
            break;
        item -= cnt;
    }
    bi = b;
    bj0 = b + item * jc;
}

__global__ void __launch_bounds__(kBlockAtoms) noalloc_pair_kernel(const NoAllocArgs a)
{
    constexpr int QS = kNoAllocQS;
    __shared__ float4 s_pos[kBlockAtoms];
    __shared__ float s_ff[QS][kMaxTypes];
    __shared__ float s_q[QS];
    __shared__ double s_red[kBlockAtoms / 32][QS];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int k0 = blockIdx.y * QS;
    for (int x = tid; x < QS * a.n_types; x += kBlockAtoms) {
        const int k = x / a.n_types, t = x - k * a.n_types;
        s_ff[k][t] = (k0 + k < a.n_q) ? a.ff[(size_t)(k0 + k) * a.n_types + t] : 0.f;
    }
    if (tid < QS)
        s_q[tid] = (k0 + tid < a.n_q) ? a.q[k0 + tid] : 0.f;
    int bi, bj0;
    decode_item(blockIdx.x, a.n_blocks, a.jchunk, bi, bj0);
    const int bj1 = min(a.n_blocks, bj0 + a.jchunk);
    const int i = bi * kBlockAtoms + tid;
    bool valid_i = i < a.n;
    const float4 pi = valid_i ? a.bodies[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const unsigned ti = __float_as_uint(pi.w);
    if (valid_i && ti >= (unsigned)a.n_types) {
        atomicOr(a.err, 1u);
        valid_i = false;
    }
    float acc[QS], comp[QS];
#pragma unroll
    for (int k = 0; k < QS; ++k) {
        acc[k] = 0.f;
        comp[k] = 0.f;
    }
    for (int b = bj0; b < bj1; ++b) {
        const int j0 = b * kBlockAtoms;
        const int jn = min(kBlockAtoms, a.n - j0);
        __syncthreads();
        if (tid < jn)
            s_pos[tid] = a.bodies[j0 + tid];
        __syncthreads();
        float S[QS];
#pragma unroll
        for (int k = 0; k < QS; ++k)
            S[k] = 0.f;
        for (int jj = 0; jj < jn; ++jj) {
            const float4 pj = s_pos[jj];
            unsigned tj = __float_as_uint(pj.w);
            bool use = valid_i && (b != bi || jj > tid);
            if (tj >= (unsigned)a.n_types) {
                if (tid == 0)
                    atomicOr(a.err, 1u);
                tj = 0;
                use = false;
            }
            float r, rinv, dx, dy, dz;
            pair_r(pi, pj, r, rinv, dx, dy, dz);
            const float sc = use ? rinv : 0.f;
#pragma unroll
            for (int k = 0; k < QS; ++k) {
                float sk, ck;
                sincos_prod(s_q[k], r, sk, ck);
                S[k] = fmaf(s_ff[k][tj], sk * sc, S[k]);
            }
        }
#pragma unroll
        for (int k = 0; k < QS; ++k)
            kahan_add(acc[k], comp[k], S[k]);
    }
    float v[QS];
#pragma unroll
    for (int k = 0; k < QS; ++k)
        v[k] = valid_i ? s_ff[k][ti] * (acc[k] - comp[k]) : 0.f;
    warp_reduce_scatter<QS>(v, lane);
    if (lane < QS)
        s_red[warp][lane] = (double)v[0];
    __syncthreads();
    if (tid < QS && k0 + tid < a.n_q) {
        double s = 0.0;
#pragma unroll
        for (int w = 0; w < kBlockAtoms / 32; ++w)
            s += s_red[w][tid];
        a.partial[(size_t)(k0 + tid) * a.n_items + blockIdx.x] = s;
    }
}

__global__ void __launch_bounds__(256) noalloc_assemble_kernel(const NoAllocArgs a)
{
    __shared__ double s_c[8], s_s[8], s_f[8];
    const int k = blockIdx.x;
    const float *row = a.ff + (size_t)k * a.n_types;
    double cross = 0.0, self = 0.0, sumf = 0.0;
    for (int x = threadIdx.x; x < a.n_items; x += blockDim.x)
        cross += a.partial[(size_t)k * a.n_items + x];
    for (int i = threadIdx.x; i < a.n; i += blockDim.x) {
        const unsigned t = __float_as_uint(a.bodies[i].w);
        const double f = t < (unsigned)a.n_types ? (double)row[t] : 0.0;
        self += f * f;
        sumf += f;
    }
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) {
        cross += __shfl_xor_sync(0xffffffffu, cross, m);
        self += __shfl_xor_sync(0xffffffffu, self, m);
        sumf += __shfl_xor_sync(0xffffffffu, sumf, m);
    }
    if ((threadIdx.x & 31) == 0) {
        s_c[threadIdx.x >> 5] = cross;
        s_s[threadIdx.x >> 5] = self;
        s_f[threadIdx.x >> 5] = sumf;
    }
    __syncthreads();
    if (threadIdx.x != 0)
        return;
    cross = self = sumf = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
        cross += s_c[w];
        self += s_s[w];
        sumf += s_f[w];
    }
    const double q = a.q[k];
    a.out[k] = (float)((q != 0.0) ? self + 2.0 * cross / q : sumf * sumf);
}

// Device address of the scratch array, looked up once per device with that
// device current (the host-side name of a __device__ array is only a
// stand-in), and again when the device's context was recreated since
// (cudaDeviceReset unloads the module; the array may then sit elsewhere).
// The context is told apart by its driver-assigned ID, read through the
// runtime's driver entry points (no link against the driver library).
static std::mutex g_setup_mu;
static double *g_scratch_addr[kMaxDevices];
static unsigned long long g_scratch_ctx[kMaxDevices];

typedef int (*CtxGetCurrentFn)(void **);
typedef int (*CtxGetIdFn)(void *, unsigned long long *);

// ID of the context current on this thread, 0 when none is current or the
// driver cannot tell (the address is then looked up again).  Called with
// g_setup_mu held.
static unsigned long long current_context_id()
{
    static bool looked_up = false;
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    if (!looked_up) {
        looked_up = true;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", (void **)&get_current, 12000,
                                             cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            get_current = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", (void **)&get_id, 12000,
                                             cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            get_id = nullptr;
    }
    void *ctx = nullptr;
    unsigned long long id = 0;
    if (get_current && get_id && get_current(&ctx) == 0 && ctx && get_id(ctx, &id) == 0)
        return id;
    return 0;
}

static rsx_status scratch_address(int dev, double **out)
{
    if (dev < 0 || dev >= kMaxDevices)
        return fail_static(RSX_INVALID_DEVICE, "device ordinal outside the supported range");
    std::lock_guard<std::mutex> lk(g_setup_mu);
    const unsigned long long ctx = current_context_id();
    if (!g_scratch_addr[dev] || ctx == 0 || ctx != g_scratch_ctx[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return fail_static(RSX_CUDA_ERROR,
                               "cudaGetSymbolAddress of the static scratch array failed");
        g_scratch_addr[dev] = static_cast<double *>(p);
        g_scratch_ctx[dev] = current_context_id(); // the lookup made the context current
    }
    *out = g_scratch_addr[dev];
    return RSX_OK;
}

} // namespace rsx

extern "C" rsx_status rsx_calc_saxs_curve_device_noalloc(const float *d_q, int n_q,
                                                         const rsx_body *d_bodies, int n_bodies,
                                                         const float *d_factors, int n_factors,
                                                         float *d_out_iq, void *stream)
{
    using namespace rsx;
    if (!d_q || !d_factors || !d_out_iq || (n_bodies > 0 && !d_bodies))
        return fail_static(RSX_INVALID_ARG, "null device pointer argument");
    if (n_q <= 0 || n_bodies < 0 || n_factors <= 0 || n_factors > kMaxTypes)
        return fail_static(RSX_INVALID_ARG, "need n_q >= 1, n_bodies >= 0, 1..32 factor types");
    const int nb = (n_bodies + kBlockAtoms - 1) / kBlockAtoms;
    const size_t cap = kNoAllocScratchDoubles - kNoAllocHeader;
    // smallest J run per item (a power of two) whose partial sums fit the array
    int jc = 1;
    long long items = (long long)nb * (nb + 1) / 2;
    while (items * n_q > (long long)cap && jc < nb) {
        jc *= 2;
        items = 0;
        for (int b = 0; b < nb; ++b)
            items += (nb - b + jc - 1) / jc;
    }
    if (items * n_q > (long long)cap)
        return fail_static(RSX_INVALID_ARG,
                           "problem too large for the 8 MiB static scratch: need "
                           "ceil(n_bodies/128) * n_q <= 1048544");
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess)
        return fail_static(RSX_INVALID_DEVICE, "no current CUDA device");
    double *scratch = nullptr;
    RSX_TRY(scratch_address(dev, &scratch));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    NoAllocArgs a;
    a.bodies = reinterpret_cast<const float4 *>(d_bodies);
    a.q = d_q;
    a.ff = d_factors;
    a.out = d_out_iq;
    a.partial = scratch + kNoAllocHeader;
    a.err = reinterpret_cast<unsigned *>(scratch);
    a.n = n_bodies;
    a.n_q = n_q;
    a.n_types = n_factors;
    a.n_blocks = nb;
    a.jchunk = jc;
    a.n_items = (int)items;
    if (cudaMemsetAsync(a.err, 0, sizeof(unsigned), st) != cudaSuccess)
        return fail_static(RSX_CUDA_ERROR, "clearing the scratch error word failed");
    if (items > 0) {
        if (inject_launch_fault())
            return fail_static(RSX_INJECTED_FAULT, "injected launch fault: no-alloc pair kernel");
        noalloc_pair_kernel<<<dim3((unsigned)items, (n_q + kNoAllocQS - 1) / kNoAllocQS),
                              kBlockAtoms, 0, st>>>(a);
        count_launch();
        if (cudaGetLastError() != cudaSuccess)
            return fail_static(RSX_CUDA_ERROR, "no-alloc pair kernel launch failed");
    }
    noalloc_assemble_kernel<<<n_q, 256, 0, st>>>(a);
    count_launch();
    if (cudaGetLastError() != cudaSuccess)
        return fail_static(RSX_CUDA_ERROR, "no-alloc assemble kernel launch failed");
    unsigned err_word = 0;
    if (cudaMemcpyAsync(&err_word, a.err, sizeof err_word, cudaMemcpyDeviceToHost, st) !=
            cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return fail_static(RSX_CUDA_ERROR, "no-alloc forward failed on the device");
    if (err_word)
        return fail_static(RSX_INVALID_ARG, "a body has a factor index >= n_factors");
    return ok();
}
