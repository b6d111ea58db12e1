/*
 * Minimal stand-in for the OpenCL C++ header, written for this project so that
 * the reference's pure-CPU host_debye.cpp compiles without an OpenCL SDK.
 * It declares only the plain value types that file and its headers use
 * (cl_float4 / cl_double4 with .s[] access, as in the Khronos headers' public
 * layout) and an empty cl::Device.  Test infrastructure only.
 */
#ifndef RSX_ORACLE_CL_SHIM_HPP
#define RSX_ORACLE_CL_SHIM_HPP
#include <cstring>
#include <string>
#include <vector>
typedef float cl_float;
typedef double cl_double;
typedef unsigned int cl_uint;
typedef int cl_int;
typedef union { cl_float s[4]; struct { cl_float x, y, z, w; }; } cl_float4;
typedef union { cl_double s[4]; struct { cl_double x, y, z, w; }; } cl_double4;
typedef cl_float4 cl_float3;
typedef cl_double4 cl_double3;
namespace cl { class Device {}; }
#endif
