// Library-level C ABI calls and host helpers of librsx.
#include "rsx_host.h"

#include <atomic>
#include <cstdio>
#include <mutex>

namespace rsx {

static thread_local std::string t_last_error;
// set by fail_static (no heap allocation); cleared by fail() and ok()
static thread_local const char *t_static_error = nullptr;
static std::mutex g_fault_mu;
static int g_fault_kind = -1;
static int g_fault_left = 0;

rsx_status fail(rsx_status st, const std::string &msg)
{
    t_static_error = nullptr;
    t_last_error = msg;
    return st;
}

rsx_status fail_static(rsx_status st, const char *msg)
{
    t_static_error = msg;
    return st;
}

rsx_status ok()
{
    t_static_error = nullptr;
    t_last_error.clear();
    return RSX_OK;
}

rsx_status cuda_status(cudaError_t e, const char *what)
{
    if (e == cudaSuccess)
        return RSX_OK;
    const rsx_status st =
        (e == cudaErrorMemoryAllocation) ? RSX_OUT_OF_MEMORY
        : (e == cudaErrorNoDevice || e == cudaErrorInvalidDevice) ? RSX_INVALID_DEVICE
        : (e == cudaErrorNoKernelImageForDevice) ? RSX_PROGRAM_NOT_LOADED
                                                 : RSX_CUDA_ERROR;
    return fail(st, std::string(what) + ": " + cudaGetErrorName(e) + " (" +
                        cudaGetErrorString(e) + ")");
}

static bool take_fault(int kind)
{
    std::lock_guard<std::mutex> lk(g_fault_mu);
    if (g_fault_kind != kind || g_fault_left <= 0)
        return false;
    if (--g_fault_left == 0) {
        g_fault_kind = -1;
        return true;
    }
    return false;
}

bool inject_alloc_fault() { return take_fault(0); }
bool inject_launch_fault() { return take_fault(1); }

rsx_status dev_alloc(void **p, size_t bytes, const char *what)
{
    *p = nullptr;
    if (inject_alloc_fault())
        return fail(RSX_INJECTED_FAULT, std::string("injected allocation fault: ") + what);
    if (bytes == 0)
        bytes = 16;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        *p = nullptr;
        return cuda_status(e, what);
    }
    return RSX_OK;
}

rsx_status host_alloc_pinned(void **p, size_t bytes, const char *what)
{
    *p = nullptr;
    if (inject_alloc_fault())
        return fail(RSX_INJECTED_FAULT, std::string("injected allocation fault: ") + what);
    if (bytes == 0)
        bytes = 16;
    cudaError_t e = cudaMallocHost(p, bytes);
    if (e != cudaSuccess) {
        *p = nullptr;
        return cuda_status(e, what);
    }
    return RSX_OK;
}

void dev_free(void *p)
{
    if (p)
        cudaFree(p);
}

void host_free_pinned(void *p)
{
    if (p)
        cudaFreeHost(p);
}

rsx_status select_device(int device, int *resolved)
{
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0)
        return fail(RSX_INVALID_DEVICE, std::string("no CUDA device available: ") +
                                            (e == cudaSuccess ? "0 devices" : cudaGetErrorString(e)));
    int dev = device;
    if (dev < 0)
        RSX_TRY_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
    if (dev >= count)
        return fail(RSX_INVALID_DEVICE, "device ordinal " + std::to_string(dev) + " out of range");
    cudaDeviceProp prop;
    RSX_TRY_CUDA(cudaGetDeviceProperties(&prop, dev), "cudaGetDeviceProperties");
    if (prop.major != 10 || prop.minor != 3)
        return fail(RSX_PROGRAM_NOT_LOADED,
                    std::string("librsx is built for sm_103a only; device ") + prop.name +
                        " is sm_" + std::to_string(prop.major) + std::to_string(prop.minor));
    *resolved = dev;
    return RSX_OK;
}

DeviceGuard::DeviceGuard(int dev)
{
    if (cudaGetDevice(&prev) != cudaSuccess)
        prev = -1;
    if (dev >= 0 && dev != prev)
        cudaSetDevice(dev);
}

DeviceGuard::~DeviceGuard()
{
    if (prev >= 0)
        cudaSetDevice(prev);
}

} // namespace rsx

extern "C" {

const char *rsx_version(void)
{
    static std::string v;
    static std::once_flag once;
    std::call_once(once, [] {
        int rt = 0;
        cudaRuntimeGetVersion(&rt);
        char buf[128];
        std::snprintf(buf, sizeof buf, "%d.%d cuda-runtime %d sm_103a", RSX_VERSION_MAJOR,
                      RSX_VERSION_MINOR, rt);
        v = buf;
    });
    return v.c_str();
}

const char *rsx_last_error(void)
{
    return rsx::t_static_error ? rsx::t_static_error : rsx::t_last_error.c_str();
}

unsigned long long rsx_launch_count(void) { return rsx::launch_count(); }

void rsx_debug_inject_fault(int kind, int nth)
{
    std::lock_guard<std::mutex> lk(rsx::g_fault_mu);
    if (nth <= 0 || (kind != 0 && kind != 1)) {
        rsx::g_fault_kind = -1;
        rsx::g_fault_left = 0;
    } else {
        rsx::g_fault_kind = kind;
        rsx::g_fault_left = nth;
    }
}

} // extern "C"
