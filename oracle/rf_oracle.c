/*
 * rf_oracle.c -- CPU oracle for the RayFactorCL tracer.  TEST INFRASTRUCTURE:
 * the checker for the CUDA library, never the thing shipped or measured as the
 * product.  Function-by-function restatement of RayFactorCL/RayFactorGPU.cl
 * ("RFG") with the op mapping stated in rf_oracle.h.  Build with
 * -O2 -ffp-contract=off (no fast-math) so that every rounding is the one the
 * source states.
 */
#include "rf_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define RFO_INF (__builtin_inff())

/* 2.0f*M_PI_F (RFG:8): twice the float nearest pi, exact in float. */
static const float RFO_2PI_F = 0x1.921fb6p+2f;

/* ------------------------------------------------------------------------ */
/* Philox4x32-10.  Published algorithm: J. Salmon, M. Moraes, R. Dror,       */
/* D. Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC'11.  The       */
/* multipliers and Weyl key increments are the published constants used by  */
/* Random123/philox.h:206-224; 10 rounds (philox.h:236).                     */
/* ------------------------------------------------------------------------ */
#define RFO_PHILOX_M0 0xD2511F53u
#define RFO_PHILOX_M1 0xCD9E8D57u
#define RFO_PHILOX_W0 0x9E3779B9u
#define RFO_PHILOX_W1 0xBB67AE85u

void rfo_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        if (r > 0) { k0 += RFO_PHILOX_W0; k1 += RFO_PHILOX_W1; }
        uint64_t p0 = (uint64_t)RFO_PHILOX_M0 * c0;
        uint64_t p1 = (uint64_t)RFO_PHILOX_M1 * c2;
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        uint32_t n1 = (uint32_t)p1;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        uint32_t n3 = (uint32_t)p0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* ------------------------------------------------------------------------ */
/* sin/cos of a float.  Method: quadrant reduction k = rint(x * 2/pi) with a  */
/* three-part Cody-Waite split of pi/2 (W. Cody, W. Waite, "Software Manual  */
/* for the Elementary Functions", 1980), then the Taylor series of sin       */
/* (to r^9) and cos (to r^10) on |r| <= pi/4 in Horner form with fmaf.       */
/* Truncation error < 3e-9 relative.  This project's CUDA code evaluates the */
/* same sequence in its own own_sincosf (csrc/rf_device.cuh), so both give   */
/* identical bits; no vendor math library is involved on either side.       */
/* ------------------------------------------------------------------------ */
static const float RFO_2_OVER_PI = 0x1.45f306p-1f;   /* float(2/pi)               */
static const float RFO_PIO2_1 = 0x1.921fb6p+0f;      /* float(pi/2)               */
static const float RFO_PIO2_2 = -0x1.777a5cp-25f;    /* float(pi/2 - PIO2_1)      */
static const float RFO_PIO2_3 = -0x1.ee59dap-50f;    /* float(pi/2 - PIO2_1 - PIO2_2) */

void rfo_sincosf(float x, float *s_out, float *c_out)
{
    const float q = rintf(x * RFO_2_OVER_PI);
    const int k = (int)q;
    float r = fmaf(-q, RFO_PIO2_1, x);
    r = fmaf(-q, RFO_PIO2_2, r);
    r = fmaf(-q, RFO_PIO2_3, r);
    const float r2 = r * r;
    /* float(1/9!), float(1/7!), float(1/5!), float(1/3!) with signs */
    float ps = fmaf(r2, 0x1.71de3ap-19f, -0x1.a01a02p-13f);
    ps = fmaf(r2, ps, 0x1.111112p-7f);
    ps = fmaf(r2, ps, -0x1.555556p-3f);
    const float sn = fmaf(r * r2, ps, r);
    /* float(1/10!), float(1/8!), float(1/6!), float(1/4!), 1/2 with signs */
    float pc = fmaf(r2, -0x1.27e4fcp-22f, 0x1.a01a02p-16f);
    pc = fmaf(r2, pc, -0x1.6c16c2p-10f);
    pc = fmaf(r2, pc, 0x1.555556p-5f);
    pc = fmaf(r2, pc, -0.5f);
    const float cs = fmaf(r2, pc, 1.0f);
    switch (k & 3) {
    case 0: *s_out = sn; *c_out = cs; break;
    case 1: *s_out = cs; *c_out = -sn; break;
    case 2: *s_out = -sn; *c_out = -cs; break;
    default: *s_out = -cs; *c_out = sn; break;
    }
}

void rfo_sincosf_array(const float *x, int64_t n, float *s, float *c)
{
    for (int64_t i = 0; i < n; ++i) rfo_sincosf(x[i], &s[i], &c[i]);
}

/* ------------------------------------------------------------------------ */
/* Streams (RFG:486-500).                                                    */
/* ------------------------------------------------------------------------ */
static void stream_bits(const rfo_params *p, int32_t emitter, int64_t gid, uint32_t u[4])
{
    uint32_t ctr[4], key[2];
    key[0] = (uint32_t)gid;            /* RFG:486 key = {gid, 0xdecafbad} */
    key[1] = p->key1;
    ctr[0] = 1u;                       /* RFG:487 + the c.v[0]++ of RFG:497 */
    if (p->compat & RFO_COMPAT_STREAMS) {
        ctr[1] = 0xf00dcafeu; ctr[2] = 0xdeadbeefu; ctr[3] = 0xbeeff00du;
    } else {
        /* outside compat mode every emitter (and scene) draws its own streams */
        ctr[1] = (uint32_t)emitter;
        ctr[2] = (uint32_t)((uint64_t)gid >> 32);
        ctr[3] = 0xbeeff00du ^ p->scene_id;
    }
    rfo_philox4x32_10(ctr, key, u);
}

/* RFG:59-62 */
static float u01_24(uint32_t u) { return (float)(u >> 8) * 0x1p-24f; }

void rfo_stream_uniforms(const rfo_params *p, int32_t emitter, int64_t gid, float out[4])
{
    uint32_t u[4];
    stream_bits(p, emitter, gid, u);
    for (int i = 0; i < 4; ++i) out[i] = u01_24(u[i]);
}

/* RFG:502-506: sub-ray v sees the uniforms rotated v+1 times by .yzwx. */
static void rotated(const float r[4], int v, float o[4])
{
    for (int i = 0; i < 4; ++i) o[i] = r[(i + v + 1) & 3];
}

/* ======================================================================== */
/* FP32 geometry                                                            */
/* ======================================================================== */
typedef struct { float x, y, z; } v3f;
typedef struct { v3f s, c; } rayf;

/* RFG:64-71 (dot -> fma chain, see rf_oracle.h) */
static v3f transform_point(const float *m, v3f p)
{
    v3f w;
    w.x = fmaf(m[3], 1.0f, fmaf(m[2], p.z, fmaf(m[1], p.y, m[0] * p.x)));
    w.y = fmaf(m[7], 1.0f, fmaf(m[6], p.z, fmaf(m[5], p.y, m[4] * p.x)));
    w.z = fmaf(m[11], 1.0f, fmaf(m[10], p.z, fmaf(m[9], p.y, m[8] * p.x)));
    return w;
}

/* RFG:73-85 */
static v3f transform_normal(const float *im, v3f n)
{
    v3f w;
    w.x = fmaf(im[0], n.x, fmaf(im[4], n.y, im[8] * n.z));
    w.y = fmaf(im[1], n.x, fmaf(im[5], n.y, im[9] * n.z));
    w.z = fmaf(im[2], n.x, fmaf(im[6], n.y, im[10] * n.z));
    const float t = 1.0f / sqrtf(fmaf(w.x, w.x, fmaf(w.y, w.y, w.z * w.z)));
    w.x *= t; w.y *= t; w.z *= t;
    return w;
}

/* RFG:87-97 */
static v3f align_dir(v3f o, v3f n)
{
    float d = 1.0f / (1.0f + n.z);
    if (isinf(d)) d = 0.5f;
    v3f w;
    w.x = n.z * o.x + n.y * d * (n.y * o.x - n.x * o.y) + n.x * o.z;
    w.y = n.x * d * (n.x * o.y - n.y * o.x) + n.z * o.y + n.y * o.z;
    w.z = -n.x * o.x - n.y * o.y + n.z * o.z;
    return w;
}

/* RFG:99-109 */
static rayf xfrm_ray(const float *im, const rayf *r)
{
    rayf o;
    o.s.x = fmaf(im[0], r->s.x, fmaf(im[1], r->s.y, fmaf(im[2], r->s.z, im[3])));
    o.c.x = fmaf(im[0], r->c.x, fmaf(im[1], r->c.y, im[2] * r->c.z));
    o.s.y = fmaf(im[4], r->s.x, fmaf(im[5], r->s.y, fmaf(im[6], r->s.z, im[7])));
    o.c.y = fmaf(im[4], r->c.x, fmaf(im[5], r->c.y, im[6] * r->c.z));
    o.s.z = fmaf(im[8], r->s.x, fmaf(im[9], r->s.y, fmaf(im[10], r->s.z, im[11])));
    o.c.z = fmaf(im[8], r->c.x, fmaf(im[9], r->c.y, im[10] * r->c.z));
    return o;
}

/* RFG:111-121 */
static v3f os_ray_direction(const float r[4])
{
    v3f o;
    float sn, cs;
    rfo_sincosf(r[2] * RFO_2PI_F, &sn, &cs);
    o.y = sn; o.x = cs;
    float t = r[3];
    o.z = sqrtf(1.0f - t);
    t = sqrtf(t);
    o.x = t * o.x;
    o.y = t * o.y;
    return o;
}

/* RFG:126-145 */
static float rectangle_hit(const float *im, const rayf *w, float eps)
{
    rayf o = xfrm_ray(im, w);
    const float th = -o.s.z * (1.0f / o.c.z);
    const float hx = fabsf(o.s.x + o.c.x * th);
    const float hy = fabsf(o.s.y + o.c.y * th);
    if (hx > 1.f || hy > 1.f || th < eps) return RFO_INF;
    return th;
}

/* RFG:147-166 */
static float disc_hit(const float *im, const rayf *w, float eps)
{
    rayf o = xfrm_ray(im, w);
    const float th = -o.s.z * (1.0f / o.c.z);
    const float hx = o.s.x + o.c.x * th;
    const float hy = o.s.y + o.c.y * th;
    const float e = hx * hx + hy * hy;
    if (e <= 1.f && th > eps) return th;
    return RFO_INF;
}

/* RFG:168-187 (util1/util2 hold squared radii, Scene.cpp:254-255) */
static float annulus_hit(const float *im, const rayf *w, float r2in, float r2out, float eps)
{
    rayf o = xfrm_ray(im, w);
    const float th = -o.s.z * (1.0f / o.c.z);
    const float hx = o.s.x + o.c.x * th;
    const float hy = o.s.y + o.c.y * th;
    const float e = fmaf(hx, hx, hy * hy);
    if (e >= r2in && e <= r2out && th > eps) return th;
    return RFO_INF;
}

/* shared root selection of RFG:206-221 / RFG:244-259 */
static float quadric_pick(const rayf *o, float t1, float t2, float eps)
{
    const float z1 = o->s.z + o->c.z * t1;
    const float z2 = o->s.z + o->c.z * t2;
    if (t1 < eps || z1 < 0.f || z1 > 1.f) t1 = RFO_INF;
    if (t2 < t1 && z2 > 0.f && z2 < 1.0f && t2 > eps) return t2;
    return t1;
}

/* RFG:189-222 (no discriminant sign check: NaN rejects) */
static float cylinder_hit(const float *im, const rayf *w, float eps)
{
    rayf o = xfrm_ray(im, w);
    const float A = fmaf(o.c.x, o.c.x, o.c.y * o.c.y);
    const float B = -fmaf(o.s.x, o.c.x, o.s.y * o.c.y);
    const float C = fmaf(o.s.x, o.s.x, fmaf(o.s.y, o.s.y, -1.f));
    const float disc = sqrtf(B * B - A * C);
    float t1, t2;
    t1 = t2 = 1.0f / A;
    t1 *= (B - disc);
    t2 *= (B + disc);
    return quadric_pick(&o, t1, t2, eps);
}

/* RFG:224-260 */
static float frustum_hit(const float *im, const rayf *w, float top, float eps)
{
    rayf o = xfrm_ray(im, w);
    const float fdir = (top - 1.0f) * o.c.z;
    const float fstart = (top - 1.0f) * o.s.z + 1.0f;
    const float A = fmaf(o.c.x, o.c.x, fmaf(o.c.y, o.c.y, -fdir * fdir));
    const float B = -fmaf(o.s.x, o.c.x, fmaf(o.s.y, o.c.y, -fstart * fdir));
    const float C = fmaf(o.s.x, o.s.x, fmaf(o.s.y, o.s.y, -fstart * fstart));
    const float disc = sqrtf(B * B - A * C);
    float t1, t2;
    t1 = t2 = 1.0f / A;
    t1 *= (B - disc);
    t2 *= (B + disc);
    return quadric_pick(&o, t1, t2, eps);
}

/* RFG:262-291.  Compat: the discriminant is used without its square root and
 * the far root is never chosen (t1 <= t2).  Default: nearest root above eps. */
static float sphere_hit(const float *im, const rayf *w, float eps, int compat)
{
    rayf o = xfrm_ray(im, w);
    const float A = o.c.x * o.c.x + o.c.y * o.c.y + o.c.z * o.c.z;
    const float B = o.c.x * o.s.x + o.c.y * o.s.y + o.c.z * o.s.z;
    const float C = o.s.x * o.s.x + o.s.y * o.s.y + o.s.z * o.s.z - 1.0f;
    if (compat) {
        float d = B * B - A * C;
        d = (d < 0.0f) ? RFO_INF : d;
        if (d > 0.f) {
            const float t1 = (-B - d) * (1.0f / A);
            const float t2 = (-B + d) * (1.0f / A);
            if (t2 < t1 && t2 > eps) return t2;
            else if (t1 > eps) return t1;
        }
        return RFO_INF;
    }
    const float d2 = B * B - A * C;
    if (!(d2 >= 0.0f)) return RFO_INF;
    const float d = sqrtf(d2);
    const float ra = 1.0f / A;
    const float t1 = (-B - d) * ra;
    const float t2 = (-B + d) * ra;
    if (t1 > eps) return t1;
    if (t2 > eps) return t2;
    return RFO_INF;
}

/* dispatch of RFG:452-460 / RFG:583-593 */
static float hit_any(int type, const float *im, float u1, float u2, const rayf *w,
                     float eps, int sphere_compat, float stale)
{
    switch (type) {
    case RFO_RECTANGLE: return rectangle_hit(im, w, eps);
    case RFO_DISC: return disc_hit(im, w, eps);
    case RFO_ANNULUS: return annulus_hit(im, w, u1, u2, eps);
    case RFO_CYLINDER: return cylinder_hit(im, w, eps);
    case RFO_SPHERE: return sphere_hit(im, w, eps, sphere_compat);
    case RFO_FRUSTUM: return frustum_hit(im, w, u1, eps);
    default: return stale; /* RFG:460: t keeps its previous value */
    }
}

/* RFG:445-472 */
static int find_object(int start, int end, const rfo_prim *pr, const rayf *w, float eps,
                       int sphere_compat)
{
    int best = -1;
    float tbest = RFO_INF, t = RFO_INF;
    for (int j = start; j < end; ++j) {
        t = hit_any(pr[j].type, pr[j].invm, pr[j].util1, pr[j].util2, w, eps, sphere_compat, t);
        if (t < tbest) { tbest = t; best = j; }
    }
    return best;
}

/* RFG:298-443: one ray from primitive e with rotated uniforms r = (x,y,z,w). */
static rayf emit(const rfo_prim *e, const float r[4])
{
    rayf ray;
    v3f p, n, o;
    float sn, cs, t;
    const v3f zn = {0.f, 0.f, 1.f};
    switch (e->type) {
    case RFO_DISC: /* RFG:298-321 */
        rfo_sincosf(r[0] * RFO_2PI_F, &sn, &cs);
        t = sqrtf(r[1]);
#ifdef RFO_PLANTED_DISC_SWAP
        /* a deliberate convention slip, compiled only by the test that shows the
         * per-ray pin against the reference kernel catches it */
        p.x = t * cs; p.y = t * sn; p.z = 0.f;
#else
        p.x = t * sn; p.y = t * cs; p.z = 0.f;
#endif
        ray.s = transform_point(e->m, p);
        o = os_ray_direction(r);
        n = transform_normal(e->invm, zn);
        ray.c = align_dir(o, n);
        break;
    case RFO_ANNULUS: /* RFG:323-345 */
        rfo_sincosf(r[0] * RFO_2PI_F, &sn, &cs);
        t = (e->util2 - e->util1) * r[1] + e->util1;
        t = sqrtf(t);
        p.x = t * sn; p.y = t * cs; p.z = 0.f;
        ray.s = transform_point(e->m, p);
        o = os_ray_direction(r);
        n = transform_normal(e->invm, zn);
        ray.c = align_dir(o, n);
        break;
    case RFO_CYLINDER: /* RFG:347-365 */
        rfo_sincosf(r[0] * RFO_2PI_F, &sn, &cs);
        p.y = sn; p.x = cs; p.z = r[1];
        ray.s = transform_point(e->m, p);
        n.x = p.x * e->util2; n.y = p.y * e->util2; n.z = 0.f;
        n = transform_normal(e->invm, n);
        o = os_ray_direction(r);
        ray.c = align_dir(o, n);
        break;
    case RFO_FRUSTUM: /* RFG:369-393 */
        p.z = (sqrtf(1.0f - r[0] + r[0] * e->util1 * e->util1) - 1.0f) * (1.0f / (e->util1 - 1.0f));
        t = 1.0f + p.z * (e->util1 - 1.0f);
        rfo_sincosf(RFO_2PI_F * r[1], &sn, &cs);
        p.y = sn; p.x = cs;
        p.x *= t; p.y *= t;
        ray.s = transform_point(e->m, p);
        n.x = p.x * e->util2;
        n.y = p.y * e->util2;
        n.z = (1.f - e->util1) * (1.f + (e->util1 - 1.f) * p.z) * e->util2;
        n = transform_normal(e->invm, n);
        o = os_ray_direction(r);
        ray.c = align_dir(o, n);
        break;
    case RFO_RECTANGLE: /* RFG:399-417 */
        p.x = 2.0f * r[0] - 1.0f; p.y = 2.0f * r[1] - 1.0f; p.z = 0.f;
        ray.s = transform_point(e->m, p);
        o = os_ray_direction(r);
        n = transform_normal(e->invm, zn);
        ray.c = align_dir(o, n);
        break;
    case RFO_SPHERE: /* RFG:419-443 */
        p.z = 2.0f * r[0] - 1.0f;
        t = sqrtf(1.0f - p.z * p.z);
        rfo_sincosf(RFO_2PI_F * r[1], &sn, &cs);
        p.y = sn; p.x = cs;
        p.x *= t; p.y *= t;
        ray.s = transform_point(e->m, p);
        n.x = p.x * e->util2; n.y = p.y * e->util2; n.z = p.z * e->util2;
        n = transform_normal(e->invm, n);
        o = os_ray_direction(r);
        ray.c = align_dir(o, n);
        break;
    default: /* RFG:516: no ray is formed; the ray stays as it was */
        memset(&ray, 0, sizeof ray);
        break;
    }
    return ray;
}

/* One full ray: runGPU body (RFG:502-525) or runBVGPU body (RFG:560-624). */
static int trace_one_f32(const rfo_prim *pr, int n, const rfo_bv *bvs, int nbv,
                         const rfo_params *p, const rayf *ray)
{
    const int sc = (p->compat & RFO_COMPAT_SPHERE) != 0;
    if (!p->use_bv) return find_object(0, n, pr, ray, p->eps, sc);
    float tbest = RFO_INF, t = RFO_INF;
    int bvi = -1, obj = -1;
    for (int w = 0; w < nbv; ++w) {
        t = hit_any(bvs[w].type, bvs[w].invm, bvs[w].util1, bvs[w].util2, ray, p->eps, sc, t);
        if (t < tbest) {
            if (bvs[w].settings == 1) {
                obj = find_object(bvs[w].objStartIndex, bvs[w].objEndIndex, pr, ray, p->eps, sc);
                if (obj != -1) { tbest = t; bvi = w; }
            } else {
                tbest = t; bvi = w;
                if (!(p->compat & RFO_COMPAT_BV_STALE)) obj = -1;
            }
        }
    }
    if (bvi != -1 && obj == -1)
        obj = find_object(bvs[bvi].objStartIndex, bvs[bvi].objEndIndex, pr, ray, p->eps, sc);
    return obj;
}

void rfo_emit_ray(const rfo_prim *prims, int32_t emitter, const rfo_params *p,
                  int64_t ray, float s[3], float c[3])
{
    float u[4], r[4];
    rfo_stream_uniforms(p, emitter, ray >> 2, u);
    rotated(u, (int)(ray & 3), r);
    rayf w = emit(&prims[emitter], r);
    s[0] = w.s.x; s[1] = w.s.y; s[2] = w.s.z;
    c[0] = w.c.x; c[1] = w.c.y; c[2] = w.c.z;
}

/* ======================================================================== */
/* FP64 twin: identical streams and control flow, double arithmetic.        */
/* ======================================================================== */
typedef struct { double x, y, z; } v3d;
typedef struct { v3d s, c; } rayd;

static const double RFO_2PI_D = 6.283185307179586476925286766559;

static v3d d_transform_point(const float *m, v3d p)
{
    v3d w;
    w.x = (double)m[0] * p.x + (double)m[1] * p.y + (double)m[2] * p.z + (double)m[3];
    w.y = (double)m[4] * p.x + (double)m[5] * p.y + (double)m[6] * p.z + (double)m[7];
    w.z = (double)m[8] * p.x + (double)m[9] * p.y + (double)m[10] * p.z + (double)m[11];
    return w;
}

static v3d d_transform_normal(const float *im, v3d n)
{
    v3d w;
    w.x = (double)im[0] * n.x + (double)im[4] * n.y + (double)im[8] * n.z;
    w.y = (double)im[1] * n.x + (double)im[5] * n.y + (double)im[9] * n.z;
    w.z = (double)im[2] * n.x + (double)im[6] * n.y + (double)im[10] * n.z;
    const double t = 1.0 / sqrt(w.x * w.x + w.y * w.y + w.z * w.z);
    w.x *= t; w.y *= t; w.z *= t;
    return w;
}

/* RFG:87-97 in FP64, with d = 1/(1 + n.z) formed as (1 - n.z)/(n.x^2 + n.y^2)
 * for a normal facing -z (equal for a unit normal; no cancellation in 1 + n.z,
 * which near -z leaves d with a few correct bits and biases the directions). */
static v3d d_align_dir(v3d o, v3d n)
{
    double d = n.z < 0.0 ? (1.0 - n.z) * (1.0 / (n.x * n.x + n.y * n.y)) : 1.0 / (1.0 + n.z);
    if (isinf(d)) d = 0.5;
    v3d w;
    w.x = n.z * o.x + n.y * d * (n.y * o.x - n.x * o.y) + n.x * o.z;
    w.y = n.x * d * (n.x * o.y - n.y * o.x) + n.z * o.y + n.y * o.z;
    w.z = -n.x * o.x - n.y * o.y + n.z * o.z;
    return w;
}

static rayd d_xfrm_ray(const float *im, const rayd *r)
{
    rayd o;
    o.s.x = (double)im[0] * r->s.x + (double)im[1] * r->s.y + (double)im[2] * r->s.z + (double)im[3];
    o.c.x = (double)im[0] * r->c.x + (double)im[1] * r->c.y + (double)im[2] * r->c.z;
    o.s.y = (double)im[4] * r->s.x + (double)im[5] * r->s.y + (double)im[6] * r->s.z + (double)im[7];
    o.c.y = (double)im[4] * r->c.x + (double)im[5] * r->c.y + (double)im[6] * r->c.z;
    o.s.z = (double)im[8] * r->s.x + (double)im[9] * r->s.y + (double)im[10] * r->s.z + (double)im[11];
    o.c.z = (double)im[8] * r->c.x + (double)im[9] * r->c.y + (double)im[10] * r->c.z;
    return o;
}

static v3d d_os_ray_direction(const float r[4])
{
    v3d o;
    const double ph = (double)r[2] * RFO_2PI_D;
    o.y = sin(ph); o.x = cos(ph);
    double t = r[3];
    o.z = sqrt(1.0 - t);
    t = sqrt(t);
    o.x *= t; o.y *= t;
    return o;
}

static double d_rectangle_hit(const float *im, const rayd *w, double eps)
{
    rayd o = d_xfrm_ray(im, w);
    const double th = -o.s.z / o.c.z;
    const double hx = fabs(o.s.x + o.c.x * th);
    const double hy = fabs(o.s.y + o.c.y * th);
    if (hx > 1.0 || hy > 1.0 || th < eps) return RFO_INF;
    return th;
}

static double d_disc_hit(const float *im, const rayd *w, double eps)
{
    rayd o = d_xfrm_ray(im, w);
    const double th = -o.s.z / o.c.z;
    const double hx = o.s.x + o.c.x * th, hy = o.s.y + o.c.y * th;
    if (hx * hx + hy * hy <= 1.0 && th > eps) return th;
    return RFO_INF;
}

static double d_annulus_hit(const float *im, const rayd *w, double a, double b, double eps)
{
    rayd o = d_xfrm_ray(im, w);
    const double th = -o.s.z / o.c.z;
    const double hx = o.s.x + o.c.x * th, hy = o.s.y + o.c.y * th;
    const double e = hx * hx + hy * hy;
    if (e >= a && e <= b && th > eps) return th;
    return RFO_INF;
}

static double d_quadric_pick(const rayd *o, double t1, double t2, double eps)
{
    const double z1 = o->s.z + o->c.z * t1;
    const double z2 = o->s.z + o->c.z * t2;
    if (t1 < eps || z1 < 0.0 || z1 > 1.0) t1 = RFO_INF;
    if (t2 < t1 && z2 > 0.0 && z2 < 1.0 && t2 > eps) return t2;
    return t1;
}

static double d_cylinder_hit(const float *im, const rayd *w, double eps)
{
    rayd o = d_xfrm_ray(im, w);
    const double A = o.c.x * o.c.x + o.c.y * o.c.y;
    const double B = -(o.s.x * o.c.x + o.s.y * o.c.y);
    const double C = o.s.x * o.s.x + o.s.y * o.s.y - 1.0;
    const double disc = sqrt(B * B - A * C);
    return d_quadric_pick(&o, (B - disc) / A, (B + disc) / A, eps);
}

static double d_frustum_hit(const float *im, const rayd *w, double top, double eps)
{
    rayd o = d_xfrm_ray(im, w);
    const double fdir = (top - 1.0) * o.c.z;
    const double fstart = (top - 1.0) * o.s.z + 1.0;
    const double A = o.c.x * o.c.x + o.c.y * o.c.y - fdir * fdir;
    const double B = -(o.s.x * o.c.x + o.s.y * o.c.y - fstart * fdir);
    const double C = o.s.x * o.s.x + o.s.y * o.s.y - fstart * fstart;
    const double disc = sqrt(B * B - A * C);
    return d_quadric_pick(&o, (B - disc) / A, (B + disc) / A, eps);
}

static double d_sphere_hit(const float *im, const rayd *w, double eps, int compat)
{
    rayd o = d_xfrm_ray(im, w);
    const double A = o.c.x * o.c.x + o.c.y * o.c.y + o.c.z * o.c.z;
    const double B = o.c.x * o.s.x + o.c.y * o.s.y + o.c.z * o.s.z;
    const double C = o.s.x * o.s.x + o.s.y * o.s.y + o.s.z * o.s.z - 1.0;
    if (compat) {
        double d = B * B - A * C;
        d = (d < 0.0) ? RFO_INF : d;
        if (d > 0.0) {
            const double t1 = (-B - d) / A, t2 = (-B + d) / A;
            if (t2 < t1 && t2 > eps) return t2;
            else if (t1 > eps) return t1;
        }
        return RFO_INF;
    }
    const double d2 = B * B - A * C;
    if (!(d2 >= 0.0)) return RFO_INF;
    const double d = sqrt(d2);
    const double t1 = (-B - d) / A, t2 = (-B + d) / A;
    if (t1 > eps) return t1;
    if (t2 > eps) return t2;
    return RFO_INF;
}

static double d_hit_any(int type, const float *im, float u1, float u2, const rayd *w,
                        double eps, int sc, double stale)
{
    switch (type) {
    case RFO_RECTANGLE: return d_rectangle_hit(im, w, eps);
    case RFO_DISC: return d_disc_hit(im, w, eps);
    case RFO_ANNULUS: return d_annulus_hit(im, w, u1, u2, eps);
    case RFO_CYLINDER: return d_cylinder_hit(im, w, eps);
    case RFO_SPHERE: return d_sphere_hit(im, w, eps, sc);
    case RFO_FRUSTUM: return d_frustum_hit(im, w, u1, eps);
    default: return stale;
    }
}

static int d_find_object(int start, int end, const rfo_prim *pr, const rayd *w, double eps, int sc)
{
    int best = -1;
    double tbest = RFO_INF, t = RFO_INF;
    for (int j = start; j < end; ++j) {
        t = d_hit_any(pr[j].type, pr[j].invm, pr[j].util1, pr[j].util2, w, eps, sc, t);
        if (t < tbest) { tbest = t; best = j; }
    }
    return best;
}

static rayd d_emit(const rfo_prim *e, const float r[4])
{
    rayd ray;
    v3d p, n, o;
    double t, ph;
    const v3d zn = {0.0, 0.0, 1.0};
    const double u1 = e->util1, u2 = e->util2;
    switch (e->type) {
    case RFO_DISC:
        ph = (double)r[0] * RFO_2PI_D;
        t = sqrt((double)r[1]);
        p.x = t * sin(ph); p.y = t * cos(ph); p.z = 0.0;
        ray.s = d_transform_point(e->m, p);
        o = d_os_ray_direction(r);
        n = d_transform_normal(e->invm, zn);
        ray.c = d_align_dir(o, n);
        break;
    case RFO_ANNULUS:
        ph = (double)r[0] * RFO_2PI_D;
        t = sqrt((u2 - u1) * (double)r[1] + u1);
        p.x = t * sin(ph); p.y = t * cos(ph); p.z = 0.0;
        ray.s = d_transform_point(e->m, p);
        o = d_os_ray_direction(r);
        n = d_transform_normal(e->invm, zn);
        ray.c = d_align_dir(o, n);
        break;
    case RFO_CYLINDER:
        ph = (double)r[0] * RFO_2PI_D;
        p.y = sin(ph); p.x = cos(ph); p.z = r[1];
        ray.s = d_transform_point(e->m, p);
        n.x = p.x * u2; n.y = p.y * u2; n.z = 0.0;
        n = d_transform_normal(e->invm, n);
        o = d_os_ray_direction(r);
        ray.c = d_align_dir(o, n);
        break;
    case RFO_FRUSTUM:
        p.z = (sqrt(1.0 - r[0] + (double)r[0] * u1 * u1) - 1.0) / (u1 - 1.0);
        t = 1.0 + p.z * (u1 - 1.0);
        ph = (double)r[1] * RFO_2PI_D;
        p.y = sin(ph) * t; p.x = cos(ph) * t;
        ray.s = d_transform_point(e->m, p);
        n.x = p.x * u2; n.y = p.y * u2; n.z = (1.0 - u1) * (1.0 + (u1 - 1.0) * p.z) * u2;
        n = d_transform_normal(e->invm, n);
        o = d_os_ray_direction(r);
        ray.c = d_align_dir(o, n);
        break;
    case RFO_RECTANGLE:
        p.x = 2.0 * r[0] - 1.0; p.y = 2.0 * r[1] - 1.0; p.z = 0.0;
        ray.s = d_transform_point(e->m, p);
        o = d_os_ray_direction(r);
        n = d_transform_normal(e->invm, zn);
        ray.c = d_align_dir(o, n);
        break;
    case RFO_SPHERE:
        p.z = 2.0 * r[0] - 1.0;
        t = sqrt(1.0 - p.z * p.z);
        ph = (double)r[1] * RFO_2PI_D;
        p.y = sin(ph) * t; p.x = cos(ph) * t;
        ray.s = d_transform_point(e->m, p);
        n.x = p.x * u2; n.y = p.y * u2; n.z = p.z * u2;
        n = d_transform_normal(e->invm, n);
        o = d_os_ray_direction(r);
        ray.c = d_align_dir(o, n);
        break;
    default:
        memset(&ray, 0, sizeof ray);
        break;
    }
    return ray;
}

static int trace_one_f64(const rfo_prim *pr, int n, const rfo_bv *bvs, int nbv,
                         const rfo_params *p, const rayd *ray)
{
    const int sc = (p->compat & RFO_COMPAT_SPHERE) != 0;
    const double eps = p->eps;
    if (!p->use_bv) return d_find_object(0, n, pr, ray, eps, sc);
    double tbest = RFO_INF, t = RFO_INF;
    int bvi = -1, obj = -1;
    for (int w = 0; w < nbv; ++w) {
        t = d_hit_any(bvs[w].type, bvs[w].invm, bvs[w].util1, bvs[w].util2, ray, eps, sc, t);
        if (t < tbest) {
            if (bvs[w].settings == 1) {
                obj = d_find_object(bvs[w].objStartIndex, bvs[w].objEndIndex, pr, ray, eps, sc);
                if (obj != -1) { tbest = t; bvi = w; }
            } else {
                tbest = t; bvi = w;
                if (!(p->compat & RFO_COMPAT_BV_STALE)) obj = -1;
            }
        }
    }
    if (bvi != -1 && obj == -1)
        obj = d_find_object(bvs[bvi].objStartIndex, bvs[bvi].objEndIndex, pr, ray, eps, sc);
    return obj;
}

/* ======================================================================== */
/* Drivers                                                                  */
/* ======================================================================== */
int32_t rfo_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

static int pick_threads(int32_t req)
{
    int mt = rfo_max_threads();
    if (req <= 0 || req > mt) return mt;
    return req;
}

static int check_args(int32_t n, int32_t nbv, const rfo_params *p, int32_t emitter)
{
    if (n <= 0 || emitter < 0 || emitter >= n) return -1;
    if (p->use_bv && nbv < 0) return -1;
    return 0;
}

/* Rays [a, b) of one emitter; one Philox draw per group of four (RFG:497-506). */
static void run_range(const rfo_prim *pr, int32_t n, const rfo_bv *bvs, int32_t nbv,
                      const rfo_params *p, int32_t emitter, int64_t a, int64_t b,
                      int32_t *hit_out, int64_t hit_base, int64_t *row, int f64)
{
    float u[4], r[4];
    int64_t cur_gid = -1;
    for (int64_t ray = a; ray < b; ++ray) {
        const int64_t gid = ray >> 2;
        if (gid != cur_gid) { rfo_stream_uniforms(p, emitter, gid, u); cur_gid = gid; }
        rotated(u, (int)(ray & 3), r);
        int h;
        if (f64) {
            rayd w = d_emit(&pr[emitter], r);
            h = trace_one_f64(pr, n, bvs, nbv, p, &w);
        } else {
            rayf w = emit(&pr[emitter], r);
            h = trace_one_f32(pr, n, bvs, nbv, p, &w);
        }
        if (hit_out) hit_out[ray - hit_base] = h;
        if (row && h >= 0) row[h] += 1;   /* RFG:522-524 */
    }
}

static int trace_rays_impl(const rfo_prim *pr, int32_t n, const rfo_bv *bvs, int32_t nbv,
                           const rfo_params *p, int32_t emitter, int64_t a, int64_t b,
                           int32_t *hit_out, int32_t nt, int f64)
{
    if (check_args(n, nbv, p, emitter) || a < 0 || b < a || !hit_out) return -1;
    const int T = pick_threads(nt);
    const int64_t total = b - a;
#pragma omp parallel num_threads(T)
    {
#ifdef _OPENMP
        const int id = omp_get_thread_num(), cnt = omp_get_num_threads();
#else
        const int id = 0, cnt = 1;
#endif
        const int64_t lo = a + total * id / cnt, hi = a + total * (id + 1) / cnt;
        run_range(pr, n, bvs, nbv, p, emitter, lo, hi, hit_out, a, NULL, f64);
    }
    return 0;
}

static int tally_impl(const rfo_prim *pr, int32_t n, const rfo_bv *bvs, int32_t nbv,
                      const rfo_params *p, int32_t emitter, int64_t n_rays, int64_t *row,
                      int32_t nt, int f64)
{
    if (check_args(n, nbv, p, emitter) || n_rays < 0 || !row) return -1;
    const int T = pick_threads(nt);
    int64_t *local = (int64_t *)calloc((size_t)T * (size_t)n, sizeof(int64_t));
    if (!local) return -2;
    const int64_t ngroups = (n_rays + 3) / 4;
#pragma omp parallel num_threads(T)
    {
#ifdef _OPENMP
        const int id = omp_get_thread_num(), cnt = omp_get_num_threads();
#else
        const int id = 0, cnt = 1;
#endif
        const int64_t g0 = ngroups * id / cnt, g1 = ngroups * (id + 1) / cnt;
        int64_t lo = g0 * 4, hi = g1 * 4;
        if (hi > n_rays) hi = n_rays;
        run_range(pr, n, bvs, nbv, p, emitter, lo, hi, NULL, 0, local + (size_t)id * n, f64);
    }
    for (int t = 0; t < T; ++t)
        for (int j = 0; j < n; ++j) row[j] += local[(size_t)t * n + j];
    free(local);
    return 0;
}

int rfo_trace_rays(const rfo_prim *prims, int32_t n, const rfo_bv *bvs, int32_t nbv,
                   const rfo_params *p, int32_t emitter, int64_t ray_begin, int64_t ray_end,
                   int32_t *hit_out, int32_t n_threads)
{
    return trace_rays_impl(prims, n, bvs, nbv, p, emitter, ray_begin, ray_end, hit_out, n_threads, 0);
}

int rfo_trace_rays_f64(const rfo_prim *prims, int32_t n, const rfo_bv *bvs, int32_t nbv,
                       const rfo_params *p, int32_t emitter, int64_t ray_begin, int64_t ray_end,
                       int32_t *hit_out, int32_t n_threads)
{
    return trace_rays_impl(prims, n, bvs, nbv, p, emitter, ray_begin, ray_end, hit_out, n_threads, 1);
}

int rfo_tally(const rfo_prim *prims, int32_t n, const rfo_bv *bvs, int32_t nbv,
              const rfo_params *p, int32_t emitter, int64_t n_rays, int64_t *row, int32_t n_threads)
{
    return tally_impl(prims, n, bvs, nbv, p, emitter, n_rays, row, n_threads, 0);
}

int rfo_tally_f64(const rfo_prim *prims, int32_t n, const rfo_bv *bvs, int32_t nbv,
                  const rfo_params *p, int32_t emitter, int64_t n_rays, int64_t *row,
                  int32_t n_threads)
{
    return tally_impl(prims, n, bvs, nbv, p, emitter, n_rays, row, n_threads, 1);
}

/* main.cpp:172-173: nthreads = rayDensity*n_samples/4 (int arithmetic), then
 * rounded to a multiple of the work-group size, halves rounding down. */
int64_t rfo_ref_nthreads(int32_t ray_density, int32_t n_samples, int32_t wg)
{
    const int64_t prod = (int64_t)ray_density * (int64_t)n_samples;
    if (prod > INT32_MAX || prod < INT32_MIN || wg <= 0) return -1;
    int64_t nt = (int64_t)((int32_t)prod / 4);
    if (nt < 0) return -1;
    const int64_t rem = nt % wg;
    return rem > wg / 2 ? nt + wg - rem : nt - rem;
}
