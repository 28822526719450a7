// rf_device.cuh -- device geometry of the tracer, templated on the arithmetic.
//
// Three arithmetic policies share one body:
//   MExact : IEEE FP32 with the op mapping of the CPU restatement
//            (mad -> fma, native_sqrt -> sqrt.rn, native_recip -> rcp.rn,
//            native_rsqrt -> rcp.rn(sqrt.rn), sincos -> own_sincosf, a*b+c in
//            the source -> separate mul and add).  Its translation unit is
//            compiled with -fmad=false, so the results are bit-identical to the
//            CPU restatement of RayFactorCL/RayFactorGPU.cl.
//   MFast  : FP32 with the hardware approximations (rcp/sqrt/rsqrt.approx and
//            __sincosf), the counterparts of OpenCL's native_* functions.
//   MF64   : the same control flow in FP64 (the FP64 tracer).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "rf_internal.h"

namespace rf {

// 2.0f * M_PI_F of RayFactorGPU.cl:8 (twice the float nearest pi).
constexpr float k2PiF = 0x1.921fb6p+2f;
constexpr double k2PiD = 6.283185307179586476925286766559;

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
// as 1, 2, 3", SC'11), the generator of Random123/philox.h that
// RayFactorGPU.cl:486-499 calls.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k)
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r) { k.x += 0x9E3779B9u; k.y += 0xBB67AE85u; }
        const uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
        const uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
    }
    return c;
}

// Stream of draw `gid` of `emitter` (RayFactorGPU.cl:486-497).  Compat mode
// keeps the reference's key {gid, key1} with a fixed counter, so every
// emitter replays the same streams; otherwise the emitter, the high word of
// gid and the scene id go into the counter.
__device__ __forceinline__ uint4 stream_bits(uint32_t compat, uint32_t key1, uint32_t scene_id,
                                             int emitter, int64_t gid)
{
    uint4 c;
    if (compat & RF_COMPAT_STREAMS)
        c = make_uint4(1u, 0xf00dcafeu, 0xdeadbeefu, 0xbeeff00du);
    else
        c = make_uint4(1u, (uint32_t)emitter, (uint32_t)((uint64_t)gid >> 32), 0xbeeff00du ^ scene_id);
    return philox4x32_10(c, make_uint2((uint32_t)gid, key1));
}

// u01_closed_open_4x32_24 (RayFactorGPU.cl:59-62): exact in FP32.
__device__ __forceinline__ float u01(uint32_t u) { return __fmul_rn(__uint2float_rn(u >> 8), 0x1p-24f); }

// sin and cos of a float: quadrant reduction k = rint(x*2/pi) with a
// three-part Cody-Waite split of pi/2 (Cody & Waite, "Software Manual for the
// Elementary Functions", 1980) and the Taylor series of sin (to r^9) and cos
// (to r^10) on |r| <= pi/4 in Horner form.  Every operation is an explicit
// round-to-nearest intrinsic, so the bits do not depend on compiler flags and
// equal the CPU restatement's.
__device__ __forceinline__ void own_sincosf(float x, float &s, float &c)
{
    const float q = rintf(__fmul_rn(x, 0x1.45f306p-1f));
    const int k = (int)q;
    float r = __fmaf_rn(-q, 0x1.921fb6p+0f, x);
    r = __fmaf_rn(-q, -0x1.777a5cp-25f, r);
    r = __fmaf_rn(-q, -0x1.ee59dap-50f, r);
    const float r2 = __fmul_rn(r, r);
    float ps = __fmaf_rn(r2, 0x1.71de3ap-19f, -0x1.a01a02p-13f);
    ps = __fmaf_rn(r2, ps, 0x1.111112p-7f);
    ps = __fmaf_rn(r2, ps, -0x1.555556p-3f);
    const float sn = __fmaf_rn(__fmul_rn(r, r2), ps, r);
    float pc = __fmaf_rn(r2, -0x1.27e4fcp-22f, 0x1.a01a02p-16f);
    pc = __fmaf_rn(r2, pc, -0x1.6c16c2p-10f);
    pc = __fmaf_rn(r2, pc, 0x1.555556p-5f);
    pc = __fmaf_rn(r2, pc, -0.5f);
    const float cs = __fmaf_rn(r2, pc, 1.0f);
    switch (k & 3) {
    case 0: s = sn; c = cs; break;
    case 1: s = cs; c = -sn; break;
    case 2: s = -sn; c = -cs; break;
    default: s = -cs; c = sn; break;
    }
}

struct MExact {
    using T = float;
    static constexpr bool kF64 = false;
    __device__ static __forceinline__ T fma(T a, T b, T c) { return __fmaf_rn(a, b, c); }
    __device__ static __forceinline__ T rcp(T x) { return __frcp_rn(x); }
    __device__ static __forceinline__ T sqrt(T x) { return __fsqrt_rn(x); }
    __device__ static __forceinline__ T rsqrt(T x) { return __frcp_rn(__fsqrt_rn(x)); }
    __device__ static __forceinline__ void sincos(T x, T &s, T &c) { own_sincosf(x, s, c); }
    __device__ static __forceinline__ T two_pi() { return k2PiF; }
    __device__ static __forceinline__ T inf() { return __int_as_float(0x7f800000); }
};

struct MFast {
    using T = float;
    static constexpr bool kF64 = false;
    __device__ static __forceinline__ T fma(T a, T b, T c) { return __fmaf_rn(a, b, c); }
    __device__ static __forceinline__ T rcp(T x)
    {
        float y;
        asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
        return y;
    }
    __device__ static __forceinline__ T sqrt(T x)
    {
        float y;
        asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
        return y;
    }
    __device__ static __forceinline__ T rsqrt(T x)
    {
        float y;
        asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
        return y;
    }
    __device__ static __forceinline__ void sincos(T x, T &s, T &c) { __sincosf(x, &s, &c); }
    __device__ static __forceinline__ T two_pi() { return k2PiF; }
    __device__ static __forceinline__ T inf() { return __int_as_float(0x7f800000); }
};

struct MF64 {
    using T = double;
    static constexpr bool kF64 = true;
    __device__ static __forceinline__ T fma(T a, T b, T c) { return __fma_rn(a, b, c); }
    __device__ static __forceinline__ T rcp(T x) { return __drcp_rn(x); }
    __device__ static __forceinline__ T sqrt(T x) { return __dsqrt_rn(x); }
    __device__ static __forceinline__ T rsqrt(T x) { return __drcp_rn(__dsqrt_rn(x)); }
    __device__ static __forceinline__ void sincos(T x, T &s, T &c) { ::sincos(x, &s, &c); }
    __device__ static __forceinline__ T two_pi() { return k2PiD; }
    __device__ static __forceinline__ T inf() { return __longlong_as_double(0x7ff0000000000000ll); }
};

template <class T> struct Ray { T sx, sy, sz, cx, cy, cz; };
template <class T> struct V3 { T x, y, z; };

// ---------------------------------------------------------------------------
// Intersection tests (RayFactorGPU.cl:99-291).  `h` is the surface's invm in
// rows r0..r2 and (type, util1, util2) in aux.
// ---------------------------------------------------------------------------
template <class M>
__device__ __forceinline__ Ray<typename M::T> xfrm_ray(const HitRec &h, const Ray<typename M::T> &w)
{
    using T = typename M::T;
    Ray<T> o;  // RayFactorGPU.cl:99-109
    o.sx = M::fma(T(h.r0.x), w.sx, M::fma(T(h.r0.y), w.sy, M::fma(T(h.r0.z), w.sz, T(h.r0.w))));
    o.cx = M::fma(T(h.r0.x), w.cx, M::fma(T(h.r0.y), w.cy, T(h.r0.z) * w.cz));
    o.sy = M::fma(T(h.r1.x), w.sx, M::fma(T(h.r1.y), w.sy, M::fma(T(h.r1.z), w.sz, T(h.r1.w))));
    o.cy = M::fma(T(h.r1.x), w.cx, M::fma(T(h.r1.y), w.cy, T(h.r1.z) * w.cz));
    o.sz = M::fma(T(h.r2.x), w.sx, M::fma(T(h.r2.y), w.sy, M::fma(T(h.r2.z), w.sz, T(h.r2.w))));
    o.cz = M::fma(T(h.r2.x), w.cx, M::fma(T(h.r2.y), w.cy, T(h.r2.z) * w.cz));
    return o;
}

template <class M>
__device__ __forceinline__ typename M::T rectangle_hit(const HitRec &h, const Ray<typename M::T> &w,
                                                       typename M::T eps)
{
    using T = typename M::T;  // RayFactorGPU.cl:126-145
    const Ray<T> o = xfrm_ray<M>(h, w);
    const T th = -o.sz * M::rcp(o.cz);
    const T hx = fabs(o.sx + o.cx * th);
    const T hy = fabs(o.sy + o.cy * th);
    if (hx > T(1) || hy > T(1) || th < eps) return M::inf();
    return th;
}

template <class M>
__device__ __forceinline__ typename M::T disc_hit(const HitRec &h, const Ray<typename M::T> &w,
                                                  typename M::T eps)
{
    using T = typename M::T;  // RayFactorGPU.cl:147-166
    const Ray<T> o = xfrm_ray<M>(h, w);
    const T th = -o.sz * M::rcp(o.cz);
    const T hx = o.sx + o.cx * th;
    const T hy = o.sy + o.cy * th;
    const T e = hx * hx + hy * hy;
    if (e <= T(1) && th > eps) return th;
    return M::inf();
}

template <class M>
__device__ __forceinline__ typename M::T annulus_hit(const HitRec &h, const Ray<typename M::T> &w,
                                                     typename M::T eps)
{
    using T = typename M::T;  // RayFactorGPU.cl:168-187 (util1/util2: squared radii)
    const Ray<T> o = xfrm_ray<M>(h, w);
    const T th = -o.sz * M::rcp(o.cz);
    const T hx = o.sx + o.cx * th;
    const T hy = o.sy + o.cy * th;
    const T e = M::fma(hx, hx, hy * hy);
    if (e >= T(h.aux.y) && e <= T(h.aux.z) && th > eps) return th;
    return M::inf();
}

template <class M>
__device__ __forceinline__ typename M::T quadric_pick(const Ray<typename M::T> &o, typename M::T t1,
                                                      typename M::T t2, typename M::T eps)
{
    using T = typename M::T;  // RayFactorGPU.cl:206-221, 244-259
    const T z1 = o.sz + o.cz * t1;
    const T z2 = o.sz + o.cz * t2;
    if (t1 < eps || z1 < T(0) || z1 > T(1)) t1 = M::inf();
    if (t2 < t1 && z2 > T(0) && z2 < T(1) && t2 > eps) return t2;
    return t1;
}

template <class M>
__device__ __forceinline__ typename M::T cylinder_hit(const HitRec &h, const Ray<typename M::T> &w,
                                                      typename M::T eps)
{
    using T = typename M::T;  // RayFactorGPU.cl:189-222
    const Ray<T> o = xfrm_ray<M>(h, w);
    const T A = M::fma(o.cx, o.cx, o.cy * o.cy);
    const T B = -M::fma(o.sx, o.cx, o.sy * o.cy);
    const T C = M::fma(o.sx, o.sx, M::fma(o.sy, o.sy, T(-1)));
    const T disc = M::sqrt(B * B - A * C);
    const T ra = M::rcp(A);
    return quadric_pick<M>(o, ra * (B - disc), ra * (B + disc), eps);
}

template <class M>
__device__ __forceinline__ typename M::T frustum_hit(const HitRec &h, const Ray<typename M::T> &w,
                                                     typename M::T eps)
{
    using T = typename M::T;  // RayFactorGPU.cl:224-260
    const Ray<T> o = xfrm_ray<M>(h, w);
    const T top = T(h.aux.y);
    const T fdir = (top - T(1)) * o.cz;
    const T fstart = (top - T(1)) * o.sz + T(1);
    const T A = M::fma(o.cx, o.cx, M::fma(o.cy, o.cy, -fdir * fdir));
    const T B = -M::fma(o.sx, o.cx, M::fma(o.sy, o.cy, -fstart * fdir));
    const T C = M::fma(o.sx, o.sx, M::fma(o.sy, o.sy, -fstart * fstart));
    const T disc = M::sqrt(B * B - A * C);
    const T ra = M::rcp(A);
    return quadric_pick<M>(o, ra * (B - disc), ra * (B + disc), eps);
}

template <class M>
__device__ __forceinline__ typename M::T sphere_hit(const HitRec &h, const Ray<typename M::T> &w,
                                                    typename M::T eps, bool compat)
{
    using T = typename M::T;  // RayFactorGPU.cl:262-291
    const Ray<T> o = xfrm_ray<M>(h, w);
    const T A = o.cx * o.cx + o.cy * o.cy + o.cz * o.cz;
    const T B = o.cx * o.sx + o.cy * o.sy + o.cz * o.sz;
    const T C = o.sx * o.sx + o.sy * o.sy + o.sz * o.sz - T(1);
    if (compat) {  // discriminant used without its square root; far root never chosen
        T d = B * B - A * C;
        d = (d < T(0)) ? M::inf() : d;
        if (d > T(0)) {
            const T t1 = (-B - d) * M::rcp(A);
            const T t2 = (-B + d) * M::rcp(A);
            if (t2 < t1 && t2 > eps) return t2;
            else if (t1 > eps) return t1;
        }
        return M::inf();
    }
    const T d2 = B * B - A * C;
    if (!(d2 >= T(0))) return M::inf();
    const T d = M::sqrt(d2);
    const T ra = M::rcp(A);
    const T t1 = (-B - d) * ra;
    const T t2 = (-B + d) * ra;
    if (t1 > eps) return t1;
    if (t2 > eps) return t2;
    return M::inf();
}

// switch of RayFactorGPU.cl:452-460; an unknown type keeps the previous t.
template <class M>
__device__ __forceinline__ typename M::T hit_any(int type, const HitRec &h, const Ray<typename M::T> &w,
                                                 typename M::T eps, bool sphere_compat,
                                                 typename M::T stale)
{
    switch (type) {
    case RF_RECTANGLE: return rectangle_hit<M>(h, w, eps);
    case RF_DISC: return disc_hit<M>(h, w, eps);
    case RF_ANNULUS: return annulus_hit<M>(h, w, eps);
    case RF_CYLINDER: return cylinder_hit<M>(h, w, eps);
    case RF_SPHERE: return sphere_hit<M>(h, w, eps, sphere_compat);
    case RF_FRUSTUM: return frustum_hit<M>(h, w, eps);
    default: return stale;
    }
}

// ---------------------------------------------------------------------------
// Emission (RayFactorGPU.cl:64-121, 298-443).
// ---------------------------------------------------------------------------
template <class M>
__device__ __forceinline__ V3<typename M::T> transform_point(const float *m, V3<typename M::T> p)
{
    using T = typename M::T;  // RayFactorGPU.cl:64-71, dot() as an fma chain
    V3<T> w;
    w.x = M::fma(T(m[3]), T(1), M::fma(T(m[2]), p.z, M::fma(T(m[1]), p.y, T(m[0]) * p.x)));
    w.y = M::fma(T(m[7]), T(1), M::fma(T(m[6]), p.z, M::fma(T(m[5]), p.y, T(m[4]) * p.x)));
    w.z = M::fma(T(m[11]), T(1), M::fma(T(m[10]), p.z, M::fma(T(m[9]), p.y, T(m[8]) * p.x)));
    return w;
}

template <class M>
__device__ __forceinline__ V3<typename M::T> transform_normal(const float *im, V3<typename M::T> n)
{
    using T = typename M::T;  // RayFactorGPU.cl:73-85
    V3<T> w;
    w.x = M::fma(T(im[0]), n.x, M::fma(T(im[4]), n.y, T(im[8]) * n.z));
    w.y = M::fma(T(im[1]), n.x, M::fma(T(im[5]), n.y, T(im[9]) * n.z));
    w.z = M::fma(T(im[2]), n.x, M::fma(T(im[6]), n.y, T(im[10]) * n.z));
    const T t = M::rsqrt(M::fma(w.x, w.x, M::fma(w.y, w.y, w.z * w.z)));
    w.x *= t;
    w.y *= t;
    w.z *= t;
    return w;
}

template <class M>
__device__ __forceinline__ V3<typename M::T> align_dir(V3<typename M::T> o, V3<typename M::T> n)
{
    using T = typename M::T;  // RayFactorGPU.cl:87-97
    // d = 1/(1 + n.z).  The FP64 tracer, which serves as the accuracy reference,
    // forms it as (1 - n.z)/(n.x^2 + n.y^2) for a normal facing -z: the same value
    // for a unit normal, without the cancellation in 1 + n.z that leaves a normal
    // 1e-7 from -z with a few correct bits (a distorted, biased rotation).
    T d = (M::kF64 && n.z < T(0)) ? (T(1) - n.z) * M::rcp(n.x * n.x + n.y * n.y) : M::rcp(T(1) + n.z);
    if (isinf(d)) d = T(0.5);
    V3<T> w;
    w.x = n.z * o.x + n.y * d * (n.y * o.x - n.x * o.y) + n.x * o.z;
    w.y = n.x * d * (n.x * o.y - n.y * o.x) + n.z * o.y + n.y * o.z;
    w.z = -n.x * o.x - n.y * o.y + n.z * o.z;
    return w;
}

template <class M>
__device__ __forceinline__ V3<typename M::T> os_ray_direction(const float r[4])
{
    using T = typename M::T;  // RayFactorGPU.cl:111-121
    V3<T> o;
    T sn, cs;
    M::sincos(T(r[2]) * M::two_pi(), sn, cs);
    o.y = sn;
    o.x = cs;
    T t = T(r[3]);
    o.z = M::sqrt(T(1) - t);
    t = M::sqrt(t);
    o.x = t * o.x;
    o.y = t * o.y;
    return o;
}

// One ray from emitter record e with the rotated uniforms r = (x, y, z, w).
template <class M>
__device__ __forceinline__ Ray<typename M::T> emit_ray(const rf_primitive &e, const float r[4])
{
    using T = typename M::T;
    V3<T> p, n, o, s, c;
    T sn, cs, t;
    const T u1 = T(e.util1), u2 = T(e.util2);
    switch (e.type) {
    case RF_DISC:  // RayFactorGPU.cl:298-321
        M::sincos(T(r[0]) * M::two_pi(), sn, cs);
        t = M::sqrt(T(r[1]));
        p.x = t * sn; p.y = t * cs; p.z = T(0);
        s = transform_point<M>(e.m, p);
        o = os_ray_direction<M>(r);
        n.x = T(0); n.y = T(0); n.z = T(1);
        n = transform_normal<M>(e.invm, n);
        c = align_dir<M>(o, n);
        break;
    case RF_ANNULUS:  // RayFactorGPU.cl:323-345
        M::sincos(T(r[0]) * M::two_pi(), sn, cs);
        t = (u2 - u1) * T(r[1]) + u1;
        t = M::sqrt(t);
        p.x = t * sn; p.y = t * cs; p.z = T(0);
        s = transform_point<M>(e.m, p);
        o = os_ray_direction<M>(r);
        n.x = T(0); n.y = T(0); n.z = T(1);
        n = transform_normal<M>(e.invm, n);
        c = align_dir<M>(o, n);
        break;
    case RF_CYLINDER:  // RayFactorGPU.cl:347-365
        M::sincos(T(r[0]) * M::two_pi(), sn, cs);
        p.y = sn; p.x = cs; p.z = T(r[1]);
        s = transform_point<M>(e.m, p);
        n.x = p.x * u2; n.y = p.y * u2; n.z = T(0);
        n = transform_normal<M>(e.invm, n);
        o = os_ray_direction<M>(r);
        c = align_dir<M>(o, n);
        break;
    case RF_FRUSTUM:  // RayFactorGPU.cl:369-393
        p.z = (M::sqrt(T(1) - T(r[0]) + T(r[0]) * u1 * u1) - T(1)) * M::rcp(u1 - T(1));
        t = T(1) + p.z * (u1 - T(1));
        M::sincos(M::two_pi() * T(r[1]), sn, cs);
        p.y = sn; p.x = cs;
        p.x *= t; p.y *= t;
        s = transform_point<M>(e.m, p);
        n.x = p.x * u2;
        n.y = p.y * u2;
        n.z = (T(1) - u1) * (T(1) + (u1 - T(1)) * p.z) * u2;
        n = transform_normal<M>(e.invm, n);
        o = os_ray_direction<M>(r);
        c = align_dir<M>(o, n);
        break;
    case RF_RECTANGLE:  // RayFactorGPU.cl:399-417
        p.x = T(2) * T(r[0]) - T(1); p.y = T(2) * T(r[1]) - T(1); p.z = T(0);
        s = transform_point<M>(e.m, p);
        o = os_ray_direction<M>(r);
        n.x = T(0); n.y = T(0); n.z = T(1);
        n = transform_normal<M>(e.invm, n);
        c = align_dir<M>(o, n);
        break;
    case RF_SPHERE:  // RayFactorGPU.cl:419-443
        p.z = T(2) * T(r[0]) - T(1);
        t = M::sqrt(T(1) - p.z * p.z);
        M::sincos(M::two_pi() * T(r[1]), sn, cs);
        p.y = sn; p.x = cs;
        p.x *= t; p.y *= t;
        s = transform_point<M>(e.m, p);
        n.x = p.x * u2; n.y = p.y * u2; n.z = p.z * u2;
        n = transform_normal<M>(e.invm, n);
        o = os_ray_direction<M>(r);
        c = align_dir<M>(o, n);
        break;
    default:
        s.x = s.y = s.z = c.x = c.y = c.z = T(0);
        break;
    }
    Ray<T> ray;
    ray.sx = s.x; ray.sy = s.y; ray.sz = s.z;
    ray.cx = c.x; ray.cy = c.y; ray.cz = c.z;
    return ray;
}

// Sub-ray v of a draw sees the uniforms rotated v+1 times by .yzwx
// (RayFactorGPU.cl:502-506).
__device__ __forceinline__ void rotate_uniforms(const float u[4], int v, float r[4])
{
#pragma unroll
    for (int i = 0; i < 4; ++i) r[i] = u[(i + v + 1) & 3];
}

// Segment of global chunk c: the last segment whose chunk_begin <= c.
__device__ __forceinline__ int find_segment(const Segment *seg, int nseg, int64_t c)
{
    int lo = 0, hi = nseg - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (seg[mid].chunk_begin <= c) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Warp-aggregated increment of bin h (h < 0: nothing) in a 32-bit histogram.
__device__ __forceinline__ void warp_tally(int *hist, int h)
{
    const unsigned peers = __match_any_sync(0xffffffffu, h);
    const int lane = threadIdx.x & 31;
    if (h >= 0 && lane == __ffs(peers) - 1) atomicAdd(&hist[h], __popc(peers));
}

__device__ __forceinline__ void warp_tally_global(unsigned long long *row, int h)
{
    const unsigned peers = __match_any_sync(0xffffffffu, h);
    const int lane = threadIdx.x & 31;
    if (h >= 0 && lane == __ffs(peers) - 1) atomicAdd(&row[h], (unsigned long long)__popc(peers));
}

}  // namespace rf
