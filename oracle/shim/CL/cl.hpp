/*
 * Minimal stand-in for the OpenCL C++ header, written for this project so that
 * the reference's pure-CPU sources (host_debye.cpp, parse_pdb.cpp, utils.cpp)
 * compile without an OpenCL SDK.  It declares the plain value types those
 * files use (cl_float4 / cl_double4 with .s[] access, as in the Khronos
 * headers' public layout) and inert cl::Platform / cl::Device objects: no
 * platform is ever reported, so the device-query code in utils.cpp compiles
 * but is never reached by the oracle.  Test infrastructure only.
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
typedef union { cl_float s[4]; struct { cl_float x, y, z, w; }; } cl_float4;
typedef union { cl_double s[4]; struct { cl_double x, y, z, w; }; } cl_double4;
typedef cl_float4 cl_float3;
typedef cl_double4 cl_double3;
enum {
    CL_DEVICE_NAME, CL_DEVICE_VENDOR, CL_DEVICE_LOCAL_MEM_TYPE, CL_LOCAL,
    CL_PLATFORM_NAME, CL_PLATFORM_VENDOR, CL_PLATFORM_VERSION
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
} // namespace cl
#endif
