// cl_compat.h -- test infrastructure.  Lets the reference's OpenCL C kernel
// source, RayFactorCL/RayFactorGPU.cl, compile as host C++ with g++ so that its
// own runGPU / runBVGPU (RayFactorGPU.cl:481-626) can be run ray by ray on the
// CPU and compared with the oracle's restatement (oracle/rf_oracle.c).
//
// oracle/build.py feeds g++ this header, then the kernel source with a few
// mechanical token rewrites (no logic is touched):
//   (float4)(a,b,c,d)          -> make_float4(a,b,c,d)     vector literal
//   v.yzwx                     -> v.yzwx()                 swizzle
//   __kernel, __global, global, __local -> removed          address spaces
//   __constant                 -> static const
// and finally ref_kernel_host.cpp, the driver.
//
// The OpenCL builtins get the fixed IEEE op mapping that the oracle and the
// bit-exact CUDA kernel share (their results are implementation-defined in
// OpenCL; this mapping is what "bit-exact" is measured against):
//   mad(a,b,c)      -> fmaf(a,b,c)
//   native_sqrt(x)  -> sqrtf(x)
//   native_recip(x) -> 1.0f / x
//   native_rsqrt(x) -> 1.0f / sqrtf(x)
//   sincos(x, &c)   -> the project's own sin/cos (rfo_sincosf, rf_oracle.c)
//   dot(a,b)        -> fmaf(a.w,b.w, fmaf(a.z,b.z, fmaf(a.y,b.y, a.x*b.x)))
// and the translation unit is compiled with -ffp-contract=off, so a source
// a*b+c keeps two roundings.
//
// Per-ray recording: each of the four sub-rays of a work-item starts with
// `rands = rands.yzwx` (RayFactorGPU.cl:506, 565), the only swizzle in the
// file, so float4::yzwx() opens a new result slot (-1 = no hit) and
// atomic_inc() (RayFactorGPU.cl:524, 623) stores the hit surface into it.
#pragma once

// Everything the kernel source and Random123 include comes first, before the
// builtin names below are defined as macros.
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <Random123/philox.h>

#include "rf_oracle.h"

// ---- vector types -----------------------------------------------------------
struct uint4 {
    uint32_t x, y, z, w;
};

struct float4 {
    float x, y, z, w;
    float4 yzwx() const;  // swizzle; also opens the next sub-ray's result slot
};

static inline float4 make_float4(float x, float y, float z, float w)
{
    float4 r;
    r.x = x; r.y = y; r.z = z; r.w = w;
    return r;
}

static inline uint4 operator>>(uint4 a, int s)
{
    uint4 r;
    r.x = a.x >> s; r.y = a.y >> s; r.z = a.z >> s; r.w = a.w >> s;
    return r;
}

static inline float4 operator*(float4 a, float b)
{
    return make_float4(a.x * b, a.y * b, a.z * b, a.w * b);
}

static inline float4 convert_float4(uint4 a)
{
    return make_float4((float)a.x, (float)a.y, (float)a.z, (float)a.w);
}

// ---- recorder state (set by the driver) --------------------------------------
struct RfclRecorder {
    int32_t *slot = nullptr;   // current sub-ray's result
    int32_t *base = nullptr;   // first result of the work-item
    int *hits = nullptr;       // the kernel's tally buffer
    int n_objects = 0;
    int from = 0;
    size_t gid = 0;
    int nslots = 0;            // sub-rays opened for the current work-item
};
static RfclRecorder g_rfcl;

inline float4 float4::yzwx() const
{
    g_rfcl.slot = g_rfcl.base + g_rfcl.nslots++;
    *g_rfcl.slot = -1;
    return make_float4(y, z, w, x);
}

// ---- builtins ---------------------------------------------------------------
static const float rfcl_M_PI_F = 3.14159265358979323846f;  // float nearest pi

static inline size_t rfcl_get_global_id(int) { return g_rfcl.gid; }

static inline int rfcl_atomic_inc(int *p)
{
    const int old = *p;
    *p = old + 1;
    *g_rfcl.slot = (int32_t)((p - g_rfcl.hits) - (ptrdiff_t)g_rfcl.from * g_rfcl.n_objects);
    return old;
}

static inline float rfcl_mad(float a, float b, float c) { return fmaf(a, b, c); }
static inline float rfcl_native_sqrt(float x) { return sqrtf(x); }
static inline float rfcl_native_recip(float x) { return 1.0f / x; }
static inline float rfcl_native_rsqrt(float x) { return 1.0f / sqrtf(x); }
static inline float rfcl_fabs(float x) { return fabsf(x); }
static inline int rfcl_isinf(float x) { return std::isinf(x) ? 1 : 0; }
static inline int rfcl_isless(float a, float b) { return a < b ? 1 : 0; }
static inline float rfcl_select(float a, float b, int c) { return c ? b : a; }

static inline float rfcl_sincos(float x, float *c)
{
    float s;
    rfo_sincosf(x, &s, c);
    return s;
}

static inline float rfcl_dot(float4 a, float4 b)
{
    return fmaf(a.w, b.w, fmaf(a.z, b.z, fmaf(a.y, b.y, a.x * b.x)));
}

#define M_PI_F rfcl_M_PI_F
#define get_global_id rfcl_get_global_id
#define atomic_inc rfcl_atomic_inc
#define mad rfcl_mad
#define native_sqrt rfcl_native_sqrt
#define native_recip rfcl_native_recip
#define native_rsqrt rfcl_native_rsqrt
#define fabs rfcl_fabs
#define isinf rfcl_isinf
#define isless rfcl_isless
#define select rfcl_select
#define sincos rfcl_sincos
#define dot rfcl_dot
