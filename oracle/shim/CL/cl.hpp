/*
 * Minimal stand-in for the OpenCL C++ header, written for this project so that
 * the reference's CPU sources (host_debye.cpp, parse_pdb.cpp, utils.cpp,
 * rsasa_cpu_alg.cpp, rsasa_algorithm.cpp) compile without an OpenCL SDK.  It
 * declares the plain value types those files use (cl_float4 / cl_double4 with
 * .s[] access, as in the Khronos headers' public layout) and inert cl::
 * objects: no platform is ever reported, and the buffer, queue, program and
 * kernel classes do nothing.  The OpenCL SASA class (rsasa_cl_gpu_alg.cpp and
 * its base re_cl_algorithm_base.cpp) is compiled against them only because
 * rsasa_algorithm.cpp's factory instantiates it; nothing here ever calls it.
 * Test infrastructure only.
 */
#ifndef RSX_ORACLE_CL_SHIM_HPP
#define RSX_ORACLE_CL_SHIM_HPP
#include <cstring>
#include <limits>
#include <ostream>
#include <string>
#include <vector>
typedef float cl_float;
typedef double cl_double;
typedef unsigned int cl_uint;
typedef int cl_int;
typedef unsigned long long cl_device_type;
typedef unsigned long long cl_mem_flags;
typedef cl_uint cl_bool;
#define CL_TRUE 1u
#define CL_FALSE 0u
#define CL_MEM_READ_WRITE (1ull << 0)
#define CL_MEM_WRITE_ONLY (1ull << 1)
#define CL_MEM_READ_ONLY (1ull << 2)
#define CL_MEM_COPY_HOST_PTR (1ull << 5)
typedef union { cl_float s[4]; struct { cl_float x, y, z, w; }; } cl_float4;
typedef union { cl_double s[4]; struct { cl_double x, y, z, w; }; } cl_double4;
typedef cl_float4 cl_float3;
typedef cl_double4 cl_double3;
enum {
    CL_DEVICE_NAME, CL_DEVICE_VENDOR, CL_DEVICE_LOCAL_MEM_TYPE, CL_LOCAL,
    CL_PLATFORM_NAME, CL_PLATFORM_VENDOR, CL_PLATFORM_VERSION,
    CL_PROGRAM_BUILD_LOG, CL_PROGRAM_BINARIES
};
#define CL_DEVICE_TYPE_CPU 2ull
#define CL_DEVICE_TYPE_GPU 4ull
#define CL_DEVICE_TYPE_ALL 0xFFFFFFFFull
namespace cl {
struct InfoValue {
    bool operator==(int) const { return false; }
};
inline std::ostream &operator<<(std::ostream &os, const InfoValue &) { return os; }
class Device {
public:
    template <int N> InfoValue getInfo(void * = nullptr) const { return {}; }
};
class Platform {
public:
    template <int N> InfoValue getInfo(void * = nullptr) const { return {}; }
    int getDevices(cl_device_type, std::vector<Device> *) const { return 0; }
    static int get(std::vector<Platform> *) { return 0; }
};
struct Error {
    const char *what() const { return "no OpenCL"; }
    int err() const { return 0; }
};
namespace detail {
template <typename T> struct KernelArgumentHandler;
}
class Context {
public:
    Context() {}
    explicit Context(const std::vector<Device> &) {}
};
class Event {};
class Buffer {
public:
    Buffer(const void * = nullptr) {}
    Buffer(const Context &, cl_mem_flags, size_t, const void *) {}
    const void *operator()() const { return nullptr; }
};
class NDRange {
public:
    NDRange() {}
    NDRange(size_t) {}
};
static const NDRange NullRange;
class Program {
public:
    typedef std::vector<std::pair<const char *, size_t>> Sources;
    Program() {}
    Program(const Context &, const Sources &) {}
    cl_int build(const std::vector<Device> &, const char * = nullptr) const { return 0; }
    template <int N> std::string getBuildInfo(const Device &) const { return std::string(); }
};
class Kernel {
public:
    Kernel() {}
    Kernel(const Program &, const char *) {}
    template <typename T> cl_int setArg(cl_uint, const T &) { return 0; }
};
class CommandQueue {
public:
    CommandQueue() {}
    CommandQueue(const Context &, const Device &) {}
    cl_int enqueueWriteBuffer(const Buffer &, cl_bool, size_t, size_t, const void *,
                              const std::vector<Event> * = nullptr, Event * = nullptr) const
    {
        return 0;
    }
    cl_int enqueueReadBuffer(const Buffer &, cl_bool, size_t, size_t, void *,
                             const std::vector<Event> * = nullptr, Event * = nullptr) const
    {
        return 0;
    }
    cl_int enqueueCopyBuffer(const Buffer &, const Buffer &, size_t, size_t, size_t,
                             const std::vector<Event> * = nullptr, Event * = nullptr) const
    {
        return 0;
    }
    cl_int enqueueNDRangeKernel(const Kernel &, const NDRange &, const NDRange &,
                                const NDRange & = NullRange,
                                const std::vector<Event> * = nullptr, Event * = nullptr) const
    {
        return 0;
    }
};
} // namespace cl
#endif
