/*
 * TEST INFRASTRUCTURE (oracle/_ref) -- not part of the engine.
 *
 * Host C++ definitions of the few OpenCL C built-ins that the reference's
 * solid-angle kernel file uses, so that the reference source compiles
 * unchanged as host code (the reference itself concatenates Random123's
 * openclfeatures.h, compilerfeatures.h, sse.h, array.h, threefry.h and the
 * kernel file into one OpenCL program, src/xmi_solid_angle_cl.c:295-323;
 * ref_cl_driver.cpp includes the same files in the same order).
 *
 * Semantics kept: float3 / uint4 component names, float overloads of the math
 * functions (std::cos(float) ... as OpenCL's float built-ins), work-item ids
 * and sizes per host thread.  Unsuffixed floating literals are double here, as
 * on an OpenCL device with fp64.
 */
#ifndef XMIMSIM_REF_CL_HOST_SHIM_H
#define XMIMSIM_REF_CL_HOST_SHIM_H

#include <climits>
#include <cmath>
#include <cstddef>
#include <cstdint>

typedef unsigned long ulong;
typedef unsigned int uint;
typedef unsigned char uchar;

#define __kernel static
#define __global
#define __constant const
#define M_PI_F 3.14159265358979323846f

using std::acos;
using std::atan;
using std::cos;
using std::fabs;
using std::sin;
using std::sqrt;

struct float3 {
  union {
    struct { float x, y, z; };
    struct { float s0, s1, s2; };
  };
  float3() : x(0.0f), y(0.0f), z(0.0f) {}
  float3(float a, float b, float c) : x(a), y(b), z(c) {}
  /* An OpenCL vector literal `(const float3) (a, b, c)` reaches C++ as a
   * cast of the comma expression, whose value is c.  The kernel file's only
   * such literal is the detector normal (0, 0, 1); any other value yields NaN
   * so that a different literal cannot pass unnoticed. */
  explicit float3(double c) : x(0.0f), y(0.0f), z(c == 1.0 ? 1.0f : NAN) {}
};

static inline float3 operator-(float3 a, float3 b) { return float3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline float3 operator+(float3 a, float3 b) { return float3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline float3 operator*(float a, float3 b) { return float3(a * b.x, a * b.y, a * b.z); }
static inline float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline float length(float3 a) { return std::sqrt(dot(a, a)); }
static inline float max(float a, float b) { return a > b ? a : b; }

struct uint4 {
  uint s0, s1, s2, s3;
};

/* work-item geometry of the host thread running the kernel body */
static thread_local size_t cl_gid[2], cl_gsize[2];
static inline size_t get_global_id(int d) { return cl_gid[d]; }
static inline size_t get_global_size(int d) { return cl_gsize[d]; }

#endif
