// Host-side helpers shared by the librsx C ABI implementation files:
// error reporting, fault injection, device buffers and pinned staging.
#pragma once
#include "../../include/rsx.h"
#include "rsx_internal.h"

#include <cuda_runtime.h>
#include <string>

namespace rsx {

// Records `msg` as this thread's last error and returns `st`.
rsx_status fail(rsx_status st, const std::string &msg);
// Records a static message (no heap allocation) and returns `st`.
rsx_status fail_static(rsx_status st, const char *msg);
// Clears the last error; returns RSX_OK.
rsx_status ok();
// Maps a CUDA error to a status (RSX_OK when e == cudaSuccess).
rsx_status cuda_status(cudaError_t e, const char *what);

// Fault injection hooks (rsx_debug_inject_fault): true when the caller must
// fail this allocation / launch.
bool inject_alloc_fault();
bool inject_launch_fault();

// Device allocation through the fault-injection hook.
rsx_status dev_alloc(void **p, size_t bytes, const char *what);
rsx_status host_alloc_pinned(void **p, size_t bytes, const char *what);
void dev_free(void *p);
void host_free_pinned(void *p);

// Device selection: `device` < 0 keeps the current one.  Verifies that a
// device exists and that it is an sm_103 part the kernels were built for.
rsx_status select_device(int device, int *resolved);

// RAII guard restoring the caller's current device.
struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev);
    ~DeviceGuard();
};

} // namespace rsx

#define RSX_TRY_CUDA(expr, what)                                                           \
    do {                                                                                   \
        cudaError_t rsx_e_ = (expr);                                                       \
        if (rsx_e_ != cudaSuccess)                                                         \
            return ::rsx::cuda_status(rsx_e_, what);                                       \
    } while (0)

#define RSX_TRY(expr)                                                                      \
    do {                                                                                   \
        rsx_status rsx_s_ = (expr);                                                        \
        if (rsx_s_ != RSX_OK)                                                              \
            return rsx_s_;                                                                 \
    } while (0)

#define RSX_LAUNCH(expr, what)                                                             \
    do {                                                                                   \
        if (::rsx::inject_launch_fault())                                                  \
            return ::rsx::fail(RSX_INJECTED_FAULT, std::string("injected launch fault: ") + \
                                                       what);                              \
        cudaError_t rsx_e_ = (expr);                                                       \
        if (rsx_e_ != cudaSuccess)                                                         \
            return ::rsx::cuda_status(rsx_e_, what);                                       \
    } while (0)
