// rf_batched.cuh -- the batched mixed-precision persistent tracing kernel.
//
// One launch traces any number of independent scenes.  Work items are chunks
// of kBatchDraws*kBatchThreads Philox draws (4 rays each) of one (scene,
// emitter) segment; a persistent grid pulls them from a device queue (an
// atomic counter), so scenes of 10 and of 400 surfaces load-balance.
//
// Per chunk (32768 rays) a block
//   1. draws every Philox word once, keeps its 24 significant bits in shared
//      memory (12 bytes per draw) and emits every ray with FP32 hardware
//      approximations (same streams and emission formulas as the plain kernel,
//      RayFactorGPU.cl:298-443) only to compute its sort key: octahedral
//      direction cell (16x16, Morton order) above a 4x4 cell of the two surface
//      parameters of the emission point,
//   2. counting-sorts the ray indices by key in shared memory,
//   3. lets its warps take packets of 32 sorted rays from a shared counter; each
//      lane re-emits its ray from the stored uniforms.  The packet's candidate
//      surfaces are the union of its rays' cell masks (built once per scene by
//      build_masks_kernel: every surface that some ray of that emitter, cell and
//      parameter patch can reach), or, for scenes without masks, the surfaces
//      whose bounding sphere the packet's origin ball and direction cone can
//      reach.  For each candidate (in index order) every lane checks its own ray
//      against the surface's bounding sphere, and the full test runs only if
//      some lane passes,
//   4. evaluates the surviving tests in FP32, with quadric discriminants in
//      cancellation-free forms; a discriminant within 16 rounding errors of
//      its terms (a grazing ray), or a cone whose A lost 12 bits, is
//      re-evaluated in FP64 after the packet, and
//   5. tallies first hits in a shared-memory row histogram (flushed as 64-bit
//      atomics whenever the (scene, emitter) row changes) straight from the
//      packet loop.
// A ray's result depends on the ray alone, never on the rays it shares a packet
// with: it is the nearest hit among the surfaces the ray's own gate admits (its
// cell mask bit and its sphere check, both functions of the ray), every one of
// which its packet tests; a lane whose packet-wide winner fails its own gate,
// or that deferred more than one test, re-traces over its gated set.  Skipping
// a surface that the ray cannot reach does not change its nearest hit; only the
// arithmetic differs from the exact kernel.  Scenes of at most kBruteMax surfaces skip
// steps 1-3: every thread tests its own rays against all surfaces.  A segment stack
// (consecutive cylinders tiling one longer cylinder, or concentric annuli in one
// plane) is one test wherever its first candidate member comes up; the member hit
// is read off the root.  The scene's tables reach shared memory by bulk copies
// (cp.async.bulk) completing on an mbarrier.
#pragma once

#include "rf_device.cuh"

namespace rf {

constexpr int kBatchThreads = 1024;
constexpr int kBatchDraws = 8;                                   // draws per thread per chunk
constexpr int kChunkDraws = kBatchThreads * kBatchDraws;         // 8192
constexpr int kChunkRays = kChunkDraws * 4;                      // 32768
constexpr int kDirGrid = 16;                                     // octahedral direction cells per axis
constexpr int kOrigCells = 16;                                   // emission-parameter cells (4 x 4)
constexpr int kCells = kDirGrid * kDirGrid * kOrigCells;         // 4096 sort keys
constexpr int kBatchHist = 512;                                  // rows up to this stay in smem
constexpr int kBruteMax = kBatchBruteMax;                        // scenes up to this are not culled
constexpr float kCondRel = 16.0f / 8388608.0f;                   // 16 ulps of the terms
constexpr float kCondA = 1.0f / 4096.0f;                         // 12 bits lost in a cone's A
static_assert(kCells == 4 * kBatchThreads, "the bucket scan gives each thread four buckets");
static_assert(kCells == kMaskCells, "one mask per sort key");
static_assert(kChunkRays <= 65536, "ray indices of a chunk are 16-bit");
constexpr int kFrameWords = kEmitFrameWords;                     // float4 words of an EmitFrame

// Rays are not stored: the lane that traces a ray re-emits it from its draw's
// uniforms, kept as 4 x 24 bits in three words (u01 uses only the top 24 bits of
// each Philox word, RayFactorGPU.cl:59-62), so a chunk costs 12 bytes per draw
// and two bytes of permutation per ray.  Until the sort the permutation array
// holds each ray's key.
struct BatchSmem {
    uint16_t perm[kChunkRays];          // key by local ray index, then sorted position -> local ray index
    uint32_t unif[3][kChunkDraws];      // the draws' 24-bit uniforms, packed
    __align__(16) int cnt[kCells];      // bucket sizes, then running bucket offsets
    int wsum[kBatchThreads / 32];
    HitRec tab[kBatchTile];
    float4 bs[kBatchTile];              // bounding spheres, squared widened radius in w
    int hist[kBatchHist];
    rf_primitive emit;
    float4 frame[kFrameWords];
    HitRec bvtab[kBatchMaxBV];          // bounding surfaces (runBVGPU semantics)
    int4 bvinfo[kBatchMaxBV];           // (settings, first child, end of children, 0)
    float4 bvbs[kBatchMaxBV];           // their bounding spheres, squared widened radius in w
    int64_t chunk;
    unsigned long long bar;             // mbarrier of the bulk copies of the scene tables
    int next_packet;
    int n_valid;
    unsigned long long work[8];
    uint32_t wcount[kBatchThreads / 32][8];  // per warp: tests by type, candidates, packets (COUNT)
};

// Bulk copies (cp.async.bulk: the TMA unit's untiled global -> shared form) of a
// scene's tables into shared memory, completing on an mbarrier.  Source and
// destination 16-byte aligned, sizes multiples of 16 (HitRec 64 B, float4 16 B).
__device__ __forceinline__ uint32_t smem_addr(const void *p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void bar_init(unsigned long long *bar)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// One thread: announce `bytes` of transfers on the barrier, then issue them.
__device__ __forceinline__ void bar_expect(unsigned long long *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, unsigned long long *bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

// Wait for the barrier's phase `parity` to complete; gives up after about 2^31
// clocks (about a second) and returns false.
__device__ __forceinline__ bool bar_wait(unsigned long long *bar, uint32_t parity)
{
    const long long t0 = clock64();
    for (;;) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(smem_addr(bar)), "r"(parity)
            : "memory");
        if (done) return true;
        if (clock64() - t0 > (1ll << 31)) return false;
    }
}

// The top 24 bits of the four Philox words of a draw in three words, and back
// as the four uniforms of u01_closed_open_4x32_24 (RayFactorGPU.cl:59-62).
__device__ __forceinline__ void pack_uniforms(uint4 u, uint32_t &w0, uint32_t &w1, uint32_t &w2)
{
    const uint32_t a = u.x >> 8, b = u.y >> 8, c = u.z >> 8, d = u.w >> 8;
    w0 = a | (b << 24);
    w1 = (b >> 8) | (c << 16);
    w2 = (c >> 16) | (d << 8);
}

__device__ __forceinline__ void unpack_uniforms(uint32_t w0, uint32_t w1, uint32_t w2, float uf[4])
{
    const uint32_t a = w0 & 0xffffffu;
    const uint32_t b = __funnelshift_r(w0, w1, 24) & 0xffffffu;
    const uint32_t c = __funnelshift_r(w1, w2, 16) & 0xffffffu;
    const uint32_t d = w2 >> 8;
    uf[0] = __fmul_rn(__uint2float_rn(a), 0x1p-24f);
    uf[1] = __fmul_rn(__uint2float_rn(b), 0x1p-24f);
    uf[2] = __fmul_rn(__uint2float_rn(c), 0x1p-24f);
    uf[3] = __fmul_rn(__uint2float_rn(d), 0x1p-24f);
}

// Emission of the mixed-precision kernels.  A planar emitter (disc, annulus,
// rectangle) has one world frame for all its rays: EmitFrame holds its origin
// and in-plane axes (the columns of m) and the rotation that alignRayDirection
// (RayFactorGPU.cl:87-97) applies to its fixed normal, all computed on the host
// in FP64 (with the FP64 tracer's cancellation-free 1 + n.z for a normal facing
// -z), so a ray costs the point's sin/cos and square root, the local direction
// and 15 multiply-adds.  Curved emitters keep the per-ray normal of emit_ray.
// frame[0] = (origin, planar flag), frame[1] = (x axis, R22), frame[2] = (y
// axis, 0), frame[3] = (R00, R01, R02, R10), frame[4] = (R11, R12, R20, R21).
__device__ __forceinline__ Ray<float> emit_mixed(const rf_primitive &e, const float4 *f, const float r[4])
{
    if (f[0].w == 0.0f) return emit_ray<MFast>(e, r);  // the same for every ray of the emitter
    float px, py, sn, cs, t;
    if (e.type == RF_RECTANGLE) {  // RayFactorGPU.cl:399-417
        px = 2.0f * r[0] - 1.0f;
        py = 2.0f * r[1] - 1.0f;
    } else {  // disc RayFactorGPU.cl:298-321, annulus :323-345
        MFast::sincos(r[0] * k2PiF, sn, cs);
        t = e.type == RF_DISC ? MFast::sqrt(r[1]) : MFast::sqrt((e.util2 - e.util1) * r[1] + e.util1);
        px = t * sn;
        py = t * cs;
    }
    const V3<float> o = os_ray_direction<MFast>(r);
    Ray<float> ray;
    ray.sx = fmaf(px, f[1].x, fmaf(py, f[2].x, f[0].x));
    ray.sy = fmaf(px, f[1].y, fmaf(py, f[2].y, f[0].y));
    ray.sz = fmaf(px, f[1].z, fmaf(py, f[2].z, f[0].z));
    ray.cx = fmaf(f[3].x, o.x, fmaf(f[3].y, o.y, f[3].z * o.z));
    ray.cy = fmaf(f[3].w, o.x, fmaf(f[4].x, o.y, f[4].y * o.z));
    ray.cz = fmaf(f[4].z, o.x, fmaf(f[4].w, o.y, f[1].w * o.z));
    return ray;
}

// Octahedral cell of a direction, kDirGrid x kDirGrid cells in Morton order.
__device__ __forceinline__ int direction_cell(float x, float y, float z)
{
    const float inv = MFast::rcp(fabsf(x) + fabsf(y) + fabsf(z) + 1e-30f);
    float u = x * inv, v = y * inv;
    if (z < 0.0f) {
        const float uu = (1.0f - fabsf(v)) * copysignf(1.0f, u);
        const float vv = (1.0f - fabsf(u)) * copysignf(1.0f, v);
        u = uu;
        v = vv;
    }
    constexpr float h = 0.5f * kDirGrid;
    const int i = min(kDirGrid - 1, max(0, (int)((u + 1.0f) * h)));
    const int j = min(kDirGrid - 1, max(0, (int)((v + 1.0f) * h)));
    static_assert(kDirGrid == 16, "4-bit Morton spread");
    // spread the 4 bits of i and j to the even / odd bits of an 8-bit code
    const int si = ((i | (i << 2)) & 0x33) | (((i | (i << 2)) & 0x33) << 1);
    const int sj = ((j | (j << 2)) & 0x33) | (((j | (j << 2)) & 0x33) << 1);
    return (si & 0x55) | ((sj & 0x55) << 1);
}

// Can the ray (origin s, direction c, idd = 1/|c|^2) reach the sphere b?  b.w
// is the squared radius, widened on the host by 1 % and for rounding.
__device__ __forceinline__ bool ray_may_hit(const Ray<float> &r, float idd, const float4 b)
{
    const float ox = b.x - r.sx, oy = b.y - r.sy, oz = b.z - r.sz;
    const float oc2 = ox * ox + oy * oy + oz * oz;
    const float bb = fmaxf(ox * r.cx + oy * r.cy + oz * r.cz, 0.0f);
    // origin inside, or the closest approach ahead of the origin is within the
    // radius (bb = 0 for a sphere behind the origin leaves the first test)
    return fmaf(-bb * bb, idd, oc2) <= b.w;
}

// Bounds of a packet of 32 rays, the same in every lane.
struct Packet {
    float ox, oy, oz, rho;  // origin ball
    float ax, ay, az;       // cone axis (unit)
    float cos_t, sin_t;     // cone half-angle
    bool cull;              // false: the cone is too wide to cull with
};

// Warp-wide float minimum / maximum in one instruction (redux.sync .f32,
// sm_100a and later); every lane gets the same, exact result.
__device__ __forceinline__ float warp_min(float v)
{
    float r;
    asm volatile("redux.sync.min.f32 %0, %1, 0xffffffff;" : "=f"(r) : "f"(v));
    return r;
}
__device__ __forceinline__ float warp_max(float v)
{
    float r;
    asm volatile("redux.sync.max.f32 %0, %1, 0xffffffff;" : "=f"(r) : "f"(v));
    return r;
}

// Bounds of a packet of rays, one per lane (lanes past the end of the chunk
// repeat the packet's first ray), the same in every lane: the origin ball is
// centred on the origins' bounding box, the cone axis on the bounding box of
// the unit directions; radius and half-angle are then exact maxima.
__device__ __forceinline__ Packet packet_bounds(const Ray<float> &r, float idd)
{
    Packet pk;
    pk.ox = 0.5f * (warp_min(r.sx) + warp_max(r.sx));
    pk.oy = 0.5f * (warp_min(r.sy) + warp_max(r.sy));
    pk.oz = 0.5f * (warp_min(r.sz) + warp_max(r.sz));
    const float dx = r.sx - pk.ox, dy = r.sy - pk.oy, dz = r.sz - pk.oz;
    // hardware square roots and reciprocals (a few ulps): the widening below and
    // the spheres' 1 % cover them
    pk.rho = MFast::sqrt(warp_max(dx * dx + dy * dy + dz * dz)) * 1.0001f + 1e-6f;
    const float ilen = MFast::sqrt(idd);
    const float nx = r.cx * ilen, ny = r.cy * ilen, nz = r.cz * ilen;
    const float ax = 0.5f * (warp_min(nx) + warp_max(nx));
    const float ay = 0.5f * (warp_min(ny) + warp_max(ny));
    const float az = 0.5f * (warp_min(nz) + warp_max(nz));
    const float al = MFast::sqrt(ax * ax + ay * ay + az * az);
    const bool ok = al > 1e-3f;
    const float ial = ok ? MFast::rcp(al) : 0.0f;
    pk.ax = ax * ial;
    pk.ay = ay * ial;
    pk.az = az * ial;
    // widened by 1e-4 for rounding in the normalisations and dot products
    const float c = warp_min(nx * pk.ax + ny * pk.ay + nz * pk.az) - 1e-4f;
    pk.cull = ok && c > 0.0f;  // cones of 90 degrees or wider are not culled
    pk.cos_t = c;
    pk.sin_t = MFast::sqrt(fmaxf(0.0f, 1.0f - c * c)) * 1.0001f;
    return pk;
}

// Can a ray starting in the packet's origin ball with a direction in its cone
// reach the sphere b (squared radius in w)?  angle(v, axis) <= theta + beta with
// sin(beta) = R/|v|, compared in cosines times |v|.
__device__ __forceinline__ bool packet_may_hit(const Packet &pk, const float4 b)
{
    if (!pk.cull) return true;
    const float vx = b.x - pk.ox, vy = b.y - pk.oy, vz = b.z - pk.oz;
    const float L2 = vx * vx + vy * vy + vz * vz;
    const float R = MFast::sqrt(b.w) * 1.0001f + pk.rho;
    const float R2 = R * R;
    if (L2 <= R2) return true;
    const float va = vx * pk.ax + vy * pk.ay + vz * pk.az;
    return va >= pk.cos_t * MFast::sqrt(L2 - R2) - pk.sin_t * R;
}

// Mixed-precision tests: FP32 with hardware approximations; quadrics whose
// discriminant is ill-conditioned are recomputed in FP64.
__device__ __forceinline__ Ray<double> to_f64(const Ray<float> &w)
{
    Ray<double> d;
    d.sx = w.sx; d.sy = w.sy; d.sz = w.sz;
    d.cx = w.cx; d.cy = w.cy; d.cz = w.cz;
    return d;
}

// The discriminants are evaluated in forms without the cancellation of B^2 -
// AC (Lagrange's identity): for the unit cylinder B^2 - AC = A - w^2 with
// w = (s x c)_z; for the cone u^2 + v^2 - w^2 with u = c_x f_s - s_x f_d,
// v = c_y f_s - s_y f_d; for the unit sphere |c|^2 - |c x s|^2.  Only a
// discriminant within 16 rounding errors of its terms (a ray grazing the
// surface) is left undecided in FP32; mag is the sum of the terms' magnitudes
// times the magnitudes that rounded in them.
__device__ __forceinline__ bool ill_conditioned(float d, float mag)
{
    return fabsf(d) < kCondRel * mag;
}

static __device__ __noinline__ float cylinder_f64(const HitRec &h, const Ray<float> &w, float eps)
{
    return (float)cylinder_hit<MF64>(h, to_f64(w), (double)eps);
}
static __device__ __noinline__ float frustum_f64(const HitRec &h, const Ray<float> &w, float eps)
{
    return (float)frustum_hit<MF64>(h, to_f64(w), (double)eps);
}
static __device__ __noinline__ float sphere_f64(const HitRec &h, const Ray<float> &w, float eps, bool sc)
{
    return (float)sphere_hit<MF64>(h, to_f64(w), (double)eps, sc);
}

// The mixed tests set `defer` instead of computing an ill-conditioned root: the
// caller re-evaluates those tests in FP64 outside its hot loop.
__device__ __forceinline__ float cylinder_mixed(const HitRec &h, const Ray<float> &w, float eps, bool &defer)
{
    const Ray<float> o = xfrm_ray<MFast>(h, w);
    const float A = fmaf(o.cx, o.cx, o.cy * o.cy);
    const float B = -fmaf(o.sx, o.cx, o.sy * o.cy);
    const float pw = o.sy * o.cx;
    const float wz = fmaf(o.sx, o.cy, -pw);
    const float d = fmaf(-wz, wz, A);
    const bool ill = ill_conditioned(d, fmaf(2.0f * fabsf(wz), fabsf(wz) + fabsf(pw), A));
    const float disc = MFast::sqrt(d);  // NaN for a miss, rejected by the comparisons
    const float ra = MFast::rcp(A);
    const float t = quadric_pick<MFast>(o, ra * (B - disc), ra * (B + disc), eps);
    defer = ill;  // selects, not a branch: the lanes of a warp stay together
    return ill ? MFast::inf() : t;
}

__device__ __forceinline__ float frustum_mixed(const HitRec &h, const Ray<float> &w, float eps, bool &defer)
{
    const Ray<float> o = xfrm_ray<MFast>(h, w);
    const float top = h.aux.y;
    const float fdir = (top - 1.f) * o.cz;
    const float fstart = (top - 1.f) * o.sz + 1.f;
    const float A = fmaf(o.cx, o.cx, fmaf(o.cy, o.cy, -fdir * fdir));
    const float B = -fmaf(o.sx, o.cx, fmaf(o.sy, o.cy, -fstart * fdir));
    // each of u, v, w is one product and one fma: rounding below eps (|p| + |x|) for
    // the product p and result x, so d is off by at most eps (3 (u^2+v^2+w^2) +
    // 2 (|u||pu| + |v||pv| + |w||pw|))
    const float pu = o.sx * fdir, pv = o.sy * fdir, pw = o.sy * o.cx;
    const float u = fmaf(o.cx, fstart, -pu);
    const float v = fmaf(o.cy, fstart, -pv);
    const float wz = fmaf(o.sx, o.cy, -pw);
    const float d = fmaf(u, u, fmaf(v, v, -wz * wz));
    const float sq = fmaf(2.0f * wz, wz, d);  // u^2 + v^2 + w^2
    const float mag = fmaf(3.0f, sq, 2.0f * fmaf(fabsf(u), fabsf(pu), fmaf(fabsf(v), fabsf(pv), fabsf(wz) * fabsf(pw))));
    const float Aterms = o.cx * o.cx + o.cy * o.cy + fdir * fdir;
    const bool ill = ill_conditioned(d, mag) || fabsf(A) < kCondA * Aterms;
    const float disc = MFast::sqrt(d);
    const float ra = MFast::rcp(A);
    const float t = quadric_pick<MFast>(o, ra * (B - disc), ra * (B + disc), eps);
    defer = ill;
    return ill ? MFast::inf() : t;
}

__device__ __forceinline__ float sphere_mixed(const HitRec &h, const Ray<float> &w, float eps, bool sc,
                                              bool &defer)
{
    if (sc) return sphere_hit<MFast>(h, w, eps, true);  // reference quirk: no root to refine
    const Ray<float> o = xfrm_ray<MFast>(h, w);
    const float A = o.cx * o.cx + o.cy * o.cy + o.cz * o.cz;
    const float B = o.cx * o.sx + o.cy * o.sy + o.cz * o.sz;
    const float kx = fmaf(o.cy, o.sz, -o.cz * o.sy);
    const float ky = fmaf(o.cz, o.sx, -o.cx * o.sz);
    const float kz = fmaf(o.cx, o.sy, -o.cy * o.sx);
    const float d2 = A - fmaf(kx, kx, fmaf(ky, ky, kz * kz));
    // near tangency |c x s| ~ |c| while its products are ~|c||s|: rounding in d2 is
    // below 2 sqrt(3) eps A |s| + eps A
    const bool ill = ill_conditioned(d2, A * fmaf(4.0f, fabsf(o.sx) + fabsf(o.sy) + fabsf(o.sz), 1.0f));
    const float d = MFast::sqrt(d2);  // NaN for a miss: both comparisons below fail
    const float ra = MFast::rcp(A);
    const float t1 = (-B - d) * ra, t2 = (-B + d) * ra;
    const float t = t1 > eps ? t1 : (t2 > eps ? t2 : MFast::inf());
    defer = ill;
    return ill ? MFast::inf() : t;
}

__device__ __forceinline__ float hit_mixed(int type, const HitRec &h, const Ray<float> &w, float eps,
                                           bool sc, bool &defer)
{
    switch (type) {
    case RF_RECTANGLE: return rectangle_hit<MFast>(h, w, eps);
    case RF_DISC: return disc_hit<MFast>(h, w, eps);
    case RF_ANNULUS: return annulus_hit<MFast>(h, w, eps);
    case RF_CYLINDER: return cylinder_mixed(h, w, eps, defer);
    case RF_FRUSTUM: return frustum_mixed(h, w, eps, defer);
    case RF_SPHERE: return sphere_mixed(h, w, eps, sc, defer);
    default: return MFast::inf();
    }
}

// FP64 evaluation of a deferred test (cold path).
static __device__ __noinline__ float hit_f64(const HitRec &h, const Ray<float> &w, float eps, bool sc)
{
    switch (__float_as_int(h.aux.x)) {
    case RF_CYLINDER: return cylinder_f64(h, w, eps);
    case RF_FRUSTUM: return frustum_f64(h, w, eps);
    case RF_SPHERE: return sphere_f64(h, w, eps, sc);
    default: return MFast::inf();
    }
}

// Segment stacks.  Consecutive cylinders [a, a + m) whose frames are one
// cylinder's shifted by whole lengths along its axis are the same quadric, so the
// index-order nearest hit among them is one cylinder test with z in [0, m] of the
// first member's frame: the near root if it lies on the stack (a root on the
// boundary of two members goes to the lower one, as the tie rule of the member
// loop does), else the far root strictly inside a member (quadric_pick rejects a
// far root on a member's rim).  ring = the member hit, 0-based.
template <class M>
__device__ __forceinline__ typename M::T stack_pick(const Ray<typename M::T> &o, typename M::T t1, typename M::T t2,
                                                    typename M::T eps, int m, int &ring)
{
    using T = typename M::T;
    const T fm = T(m);
    const T z1 = o.sz + o.cz * t1;
    const T z2 = o.sz + o.cz * t2;
    const bool v1 = !(t1 < eps || z1 < T(0) || z1 > fm);
    const T f2 = floor(z2);
    const bool v2 = t2 > eps && z2 > T(0) && z2 < fm && z2 != f2;
    const int r1 = z1 > T(0) ? (int)ceil(z1) - 1 : 0;
    ring = min(m - 1, max(0, v1 ? r1 : (int)f2));
    return v1 ? t1 : (v2 ? t2 : M::inf());
}

__device__ __forceinline__ float stack_mixed(const HitRec &h, const Ray<float> &w, float eps, bool &defer, int &ring)
{
    const Ray<float> o = xfrm_ray<MFast>(h, w);  // as cylinder_mixed
    const float A = fmaf(o.cx, o.cx, o.cy * o.cy);
    const float B = -fmaf(o.sx, o.cx, o.sy * o.cy);
    const float pw = o.sy * o.cx;
    const float wz = fmaf(o.sx, o.cy, -pw);
    const float d = fmaf(-wz, wz, A);
    const bool ill = ill_conditioned(d, fmaf(2.0f * fabsf(wz), fabsf(wz) + fabsf(pw), A));
    const float disc = MFast::sqrt(d);
    const float ra = MFast::rcp(A);
    const float t = stack_pick<MFast>(o, ra * (B - disc), ra * (B + disc), eps, (int)h.aux.y, ring);
    defer = ill;
    return ill ? MFast::inf() : t;
}

static __device__ __noinline__ float stack_f64(const HitRec &h, const Ray<float> &w, float eps, int &ring)
{
    using T = double;  // as cylinder_hit<MF64>
    const Ray<T> o = xfrm_ray<MF64>(h, to_f64(w));
    const T A = MF64::fma(o.cx, o.cx, o.cy * o.cy);
    const T B = -MF64::fma(o.sx, o.cx, o.sy * o.cy);
    const T C = MF64::fma(o.sx, o.sx, MF64::fma(o.sy, o.sy, T(-1)));
    const T disc = MF64::sqrt(B * B - A * C);
    const T ra = MF64::rcp(A);
    return (float)stack_pick<MF64>(o, ra * (B - disc), ra * (B + disc), (T)eps, (int)h.aux.y, ring);
}

// First member of the stack that surface j (a member, record h) belongs to, and
// one past its last.
__device__ __forceinline__ int stack_first(const HitRec &h, int j) { return j - (__float_as_int(h.aux.w) & 0xffff); }
__device__ __forceinline__ int stack_count(const HitRec &h) { return (int)((unsigned)__float_as_int(h.aux.w) >> 16); }
__device__ __forceinline__ int stack_end(const HitRec &h, int j) { return stack_first(h, j) + stack_count(h); }
__device__ __forceinline__ bool is_stack(int type) { return type >= kStackType; }
// The work counters' type of a test: a stack's members' own.
__device__ __forceinline__ int stat_type(int type)
{
    return type == kStackType ? RF_CYLINDER : (type == kPlateType ? RF_ANNULUS : type);
}

// A plate: concentric annuli [a, a + m) in one plane and frame, each one's outer
// squared radius (util2) the next one's inner (util1), bit for bit.  The plane is
// hit once with annulus_hit's arithmetic; the member is the lowest whose
// [util1, util2] holds e = |hit|^2 (a shared rim goes to the lower member, as the
// member loop's tie rule gives), found by a binary search over the members'
// util2 (tab: the scene's records, shared memory when resident).  The same
// arithmetic as testing the members one by one, so the same result.
__device__ __forceinline__ float plate_mixed(const HitRec &h, int j, const HitRec *tab, bool resident,
                                             const Ray<float> &w, float eps, int &idx)
{
    const Ray<float> o = xfrm_ray<MFast>(h, w);
    const float th = -o.sz * MFast::rcp(o.cz);
    const float hx = o.sx + o.cx * th;
    const float hy = o.sy + o.cy * th;
    const float e = MFast::fma(hx, hx, hy * hy);
    const int a = stack_first(h, j);
    auto util2 = [&](int k) { return resident ? tab[a + k].aux.z : __ldg(&tab[a + k].aux.z); };
    int base = 0, len = stack_count(h);  // lowest k with util2_k >= e (uniform trip count)
    while (len > 1) {
        const int half = len >> 1;
        base = util2(base + half - 1) < e ? base + half : base;
        len -= half;
    }
    const float lo = resident ? tab[a].aux.y : __ldg(&tab[a].aux.y);
    idx = a + base;
    return (e >= lo && e <= util2(base) && th > eps) ? th : MFast::inf();
}

// The mixed test of surface j (record h) -- for a stack member, the stack's --
// with idx the surface hit (j, or the member of the stack); tab, resident: the
// scene's records, for plates.
template <bool STK>
__device__ __forceinline__ float test_mixed(int type, const HitRec &h, int j, const HitRec *tab, bool resident,
                                            const Ray<float> &w, float eps, bool sc, bool &defer, int &idx)
{
    if (STK && type == kStackType) {
        int ring;
        const float t = stack_mixed(h, w, eps, defer, ring);
        idx = stack_first(h, j) + ring;
        return t;
    }
    if (STK && type == kPlateType) return plate_mixed(h, j, tab, resident, w, eps, idx);
    idx = j;
    return hit_mixed(type, h, w, eps, sc, defer);
}

// FP64 evaluation of a deferred test of surface j, idx as in test_mixed.
template <bool STK>
__device__ __forceinline__ float test_f64(const HitRec &h, int j, const Ray<float> &w, float eps, bool sc, int &idx)
{
    if (STK && __float_as_int(h.aux.x) == kStackType) {
        int ring;
        const float t = stack_f64(h, w, eps, ring);
        idx = stack_first(h, j) + ring;
        return t;
    }
    idx = j;
    return hit_f64(h, w, eps, sc);
}

// Sort key of a ray: its direction cell above the 4 x 4 cell of the two surface
// parameters (r[0], r[1]) of its emission point.
__device__ __forceinline__ int ray_key(const Ray<float> &ray, const float r[4])
{
    return (direction_cell(ray.cx, ray.cy, ray.cz) << 4) | (min(3, (int)(r[0] * 4.0f)) << 2) |
           min(3, (int)(r[1] * 4.0f));
}

// A planar emitter (disc, annulus, rectangle) cannot be hit by its own rays:
// they leave its plane into the open half-space of its normal (o.z =
// sqrt(1 - r[3]) >= 2^-12, RayFactorGPU.cl:115), so t = 0 is the only
// intersection; an FP32 "self-hit" further on is rounding (the FP64 tracer has
// none).  The mixed kernels skip that test; -1 = nothing to skip.
__device__ __forceinline__ int self_skip(const rf_primitive &e, int emitter)
{
    return (e.type == RF_DISC || e.type == RF_ANNULUS || e.type == RF_RECTANGLE) ? emitter : -1;
}

// The lane's own gate for surface j: its cell's mask bit (when the scene has
// masks) and its ray's bounding-sphere check.
__device__ __forceinline__ bool own_gate(const uint32_t *mcell, int j, const Ray<float> &ray, float idd,
                                         const float4 b)
{
    if (mcell && !((__ldg(mcell + (j >> 5)) >> (j & 31)) & 1u)) return false;
    return ray_may_hit(ray, idd, b);
}

// Bits of a 32-surface candidate word from position k on (k <= 0: all, k >= 32: none).
__device__ __forceinline__ unsigned keep_from(int k)
{
    return k <= 0 ? ~0u : (k >= 32 ? 0u : (~0u << k));
}

// The candidate loop's test: hit_mixed's, plus segment stacks.  idx (j on entry)
// gets the surface hit; a stack's other members leave the candidate word cm and
// the pair's second candidate (vb = 0 when jb is one): skip_to = one past the
// stack, for later words.
__device__ __forceinline__ float hit_hot(int type, const HitRec &h, int j, const HitRec *tab, bool resident,
                                         const Ray<float> &w, float eps, bool sc, bool &defer, int &idx, int jw,
                                         unsigned &cm, int &skip_to, int jb, unsigned &vb)
{
    switch (type) {
    case RF_RECTANGLE: return rectangle_hit<MFast>(h, w, eps);
    case RF_DISC: return disc_hit<MFast>(h, w, eps);
    case RF_ANNULUS: return annulus_hit<MFast>(h, w, eps);
    case RF_CYLINDER: return cylinder_mixed(h, w, eps, defer);
    case RF_FRUSTUM: return frustum_mixed(h, w, eps, defer);
    case RF_SPHERE: return sphere_mixed(h, w, eps, sc, defer);
    case kStackType: {
        int ring;
        const float t = stack_mixed(h, w, eps, defer, ring);
        idx = stack_first(h, j) + ring;
        skip_to = stack_end(h, j);
        cm &= keep_from(skip_to - jw);
        if (jb < skip_to) vb = 0u;
        return t;
    }
    case kPlateType: {
        const float t = plate_mixed(h, j, tab, resident, w, eps, idx);
        skip_to = stack_end(h, j);
        cm &= keep_from(skip_to - jw);
        if (jb < skip_to) vb = 0u;
        return t;
    }
    default: return MFast::inf();
    }
}

// Full nearest-hit search for one ray over the surfaces [lo, hi) its gate admits
// (gated: the cell mask when mcell is set, and the bounding-sphere check; else
// every surface but skip), with FP64 for every ill-conditioned quadric; nf64
// counts the FP64 evaluations.  Cold path: rays that deferred a test they could
// not resolve in their hot loop.
template <bool STK>
static __device__ __noinline__ int retrace_f64(int lo, int hi, bool resident, const HitRec *stab, const HitRec *gtab,
                                        const float4 *sbs, const float4 *gbs, const uint32_t *mcell, bool gated,
                                        const Ray<float> &ray, float idd, float eps, bool sc, int skip, int &nf64)
{
    float tb = MFast::inf();
    int bi = -1;
    for (int j = lo; j < hi; ++j) {
        if (j == skip) continue;
        if (gated && !own_gate(mcell, j, ray, idd, resident ? sbs[j] : __ldg(gbs + j))) continue;
        const HitRec h = resident ? stab[j] : load_rec(gtab, j);
        const int type = __float_as_int(h.aux.x);
        bool defer = false;
        int idx;
        float t = test_mixed<STK>(type, h, j, resident ? stab : gtab, resident, ray, eps, sc, defer, idx);
        if (defer) {
            t = test_f64<STK>(h, j, ray, eps, sc, idx);
            ++nf64;
        }
        if (t < tb) { tb = t; bi = idx; }
        if (STK && is_stack(type)) j = stack_end(h, j) - 1;  // one test for the whole stack
    }
    return bi;
}

// Nearest hit of a ray tested against every surface of [lo, hi) but skip, in
// index order: bi from the hot loop, deferred whether it deferred any test; such
// a ray is traced again with FP64 for each deferred test.  Shared by the
// small-scene paths of the batched kernel and of mixed_small_kernel, so both
// give the same result.
template <bool STK>
__device__ __forceinline__ int resolve_brute(int bi, bool deferred, int lo, int hi, bool resident,
                                             const HitRec *stab, const HitRec *gtab, const Ray<float> &ray,
                                             float eps, bool sc, int skip, int &nref)
{
    if (deferred)
        bi = retrace_f64<STK>(lo, hi, resident, stab, gtab, nullptr, nullptr, nullptr, false, ray, 0.0f, eps, sc, skip,
                         nref);
    return bi;
}

// The bounding-surface walk of runBVGPU (RayFactorGPU.cl:580-619) for one ray:
// surfaces w = 0..nbv-1 in order, each tested in mixed precision (FP64 when
// ill-conditioned); find(lo, hi) is the ray's nearest hit among the children
// [lo, hi) (findObject, :445-472).  bvbs: the surfaces' bounding spheres.  A ray
// needs its children's hit only when w is nearer than its best so far, so find()
// runs only then: WARP (find() is
// warp-wide, every lane here): when that holds in some lane of the warp, in
// every lane, so the warp-wide steps stay in step; else per lane.  stale:
// RF_COMPAT_BV_STALE, where a plain bounding surface that becomes the nearest
// keeps the child found under an earlier one (:596-619).
template <bool WARP, class Find>
__device__ __forceinline__ int bv_select(const HitRec *bvtab, const int4 *bvinfo, const float4 *bvbs, int nbv,
                                         const Ray<float> &ray, float eps, bool sc, bool stale, Find find)
{
    float tbest = MFast::inf();
    int bvi = -1, obj = -1, nb = -1;  // nb: children's nearest hit of the current winner bvi
    const float idd = MFast::rcp(ray.cx * ray.cx + ray.cy * ray.cy + ray.cz * ray.cz);
    for (int w = 0; w < nbv; ++w) {
        // a ray that cannot reach w's bounding sphere misses w (t = inf: nothing changes);
        // the warp skips w when that holds in every lane
        const bool may = ray_may_hit(ray, idd, bvbs[w]);
        if (WARP ? !__any_sync(0xffffffffu, may) : !may) continue;
        const HitRec hb = bvtab[w];
        bool defer = false;
        float t = hit_mixed(__float_as_int(hb.aux.x), hb, ray, eps, sc, defer);
        if (defer) t = hit_f64(hb, ray, eps, sc);
        const int4 info = bvinfo[w];
        const bool nearer = t < tbest;
        const bool run = WARP ? __any_sync(0xffffffffu, nearer) : nearer;
        const int nw = run ? find(info.y, info.z) : -1;  // used only when nearer
        if (nearer) {
            if (info.x == 1) {  // test the children at once; the surface counts only if one is hit
                obj = nw;
                if (nw != -1) { tbest = t; bvi = w; nb = nw; }
            } else {
                tbest = t;
                bvi = w;
                nb = nw;
                if (!stale) obj = -1;
            }
        }
    }
    if (bvi != -1 && obj == -1) obj = nb;  // the winner's children
    return obj;
}

// RESIDENT: every scene of the launch fits the shared-memory tables
// (n <= kBatchTile); otherwise surfaces are read through L1.  COUNT: also count
// the tests by surface type, the candidates and the packets (p.work); the
// counters cost a few per cent, so timed runs leave them out.  BV: one resident
// scene with bounding surfaces (p.bvtab, p.bvinfo, p.nbv <= kBatchMaxBV) traced
// with runBVGPU's semantics (bv_select).  STK: some scene has segment stacks
// (kStackType records); the candidate loops then test a stack once.
template <bool REC, bool RESIDENT, bool COUNT, bool BV, bool STK>
__global__ void __launch_bounds__(kBatchThreads, 1) batched_kernel(const TraceParams p)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    BatchSmem &S = *reinterpret_cast<BatchSmem *>(smem_raw);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const bool sc = (p.compat & RF_COMPAT_SPHERE) != 0;
    float eps = p.eps;  // the current scene's (SceneInfo::eps)
    const int64_t total = p.d_total ? *p.d_total : p.total_chunks;
    const int nseg = p.d_nseg ? *p.d_nseg : p.nseg;

    int cur_scene = -1, cur_emitter = -1;
    SceneInfo si{};
    int nref = 0;
    if (COUNT) {
        if (tid < 8) S.work[tid] = 0ull;
        if (lane < 8) S.wcount[warp][lane] = 0u;
    }
    bool hist_on = false;
    int row_chunks = 0;   // chunks tallied into the shared-memory row since its last flush
    uint32_t tcount = 0;  // COUNT, lane t < 6: lane-tests of surfaces of type t by this warp (this chunk)
    const uint32_t *mrow = nullptr;  // cell masks of the current row (null: packet bounds instead)
    uint32_t bar_parity = 0;         // phase of S.bar the next table copy completes
    if (RESIDENT && tid == 0) bar_init(&S.bar);  // visible after the chunk loop's first barrier

    auto flush = [&]() {
        __syncthreads();
        if (hist_on && cur_emitter >= 0) {
            unsigned long long *row = p.hits + si.hits_off + (int64_t)cur_emitter * si.n;
            for (int i = tid; i < si.n; i += blockDim.x) {
                const int v = S.hist[i];
                if (v) {
                    atomicAdd(row + i, (unsigned long long)v);
                    S.hist[i] = 0;
                }
            }
        }
        __syncthreads();
    };
    auto fold_counts = [&]() {
        if (COUNT) {
            if (lane < 6) S.wcount[warp][lane] += tcount;
            tcount = 0;
            __syncwarp();
            if (lane < 8) {
                const uint32_t v = S.wcount[warp][lane];
                if (v) atomicAdd(&S.work[lane], (unsigned long long)v);
                S.wcount[warp][lane] = 0u;
            }
        }
    };

    for (;;) {
        if (tid == 0) S.chunk = (int64_t)atomicAdd(p.queue, 1ull);
        __syncthreads();
        const int64_t c = S.chunk;
        if (c >= total) break;  // block-uniform
        const int s = find_segment(p.seg, nseg, c);
        const Segment sg = p.seg[s];

        if (!REC && hist_on && ++row_chunks >= 32768) {  // keep the 32-bit bins far from overflow
            flush();                                     // (at most 32768 hits per bin per chunk)
            row_chunks = 0;
        }
        bool staged = false;  // RESIDENT: this chunk copies a new scene's tables
        if (sg.scene != cur_scene || sg.emitter != cur_emitter) {
            if (!REC) flush();
            row_chunks = 0;
            if (sg.scene != cur_scene) {
                si = p.scenes[sg.scene];
                eps = si.eps;
                hist_on = !REC && si.n <= kBatchHist;
                if (hist_on)
                    for (int i = tid; i < si.n; i += blockDim.x) S.hist[i] = 0;
                if (RESIDENT) {  // resident tables: two bulk copies, waited for below
                    // (every thread finished with the previous tables before the chunk's barrier)
                    if (tid == 0) {
                        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                        const uint32_t tb = (uint32_t)(sizeof(HitRec) * si.n), sb = (uint32_t)(sizeof(float4) * si.n);
                        bar_expect(&S.bar, tb + sb);
                        bulk_load(S.tab, p.tab + si.prim_off, tb, &S.bar);
                        bulk_load(S.bs, p.bsph + si.prim_off, sb, &S.bar);
                    }
                    staged = true;
                }
                if (BV) {
                    for (int i = tid; i < 4 * p.nbv; i += blockDim.x)
                        reinterpret_cast<float4 *>(S.bvtab)[i] = __ldg(reinterpret_cast<const float4 *>(p.bvtab) + i);
                    for (int i = tid; i < p.nbv; i += blockDim.x) {
                        S.bvinfo[i] = __ldg(p.bvinfo + i);
                        S.bvbs[i] = __ldg(p.bvsph + i);
                    }
                }
                cur_scene = sg.scene;
            }
            if (tid < (int)(sizeof(rf_primitive) / 4))
                reinterpret_cast<float *>(&S.emit)[tid] =
                    reinterpret_cast<const float *>(p.emit + si.prim_off + sg.emitter)[tid];
            if (tid < kFrameWords) S.frame[tid] = p.frame[(int64_t)(si.prim_off + sg.emitter) * kFrameWords + tid];
            cur_emitter = sg.emitter;
            mrow = nullptr;
            if (p.mask_off) {
                const int64_t mo = p.mask_off[si.prim_off + sg.emitter];
                if (mo >= 0) mrow = p.cmask + mo;
            }
        }
        if (RESIDENT && staged) {  // block-uniform: every thread waits for the copies
            const bool ok = bar_wait(&S.bar, bar_parity);
            if (__syncthreads_or(!ok)) {  // gave up: flag it, let the copies land (bounded), stop
                if (!ok) bar_wait(&S.bar, bar_parity);
                if (tid == 0 && p.err) atomicExch(p.err, 3);
                return;
            }
            bar_parity ^= 1u;
        }
        for (int i = tid; i < kCells; i += blockDim.x) S.cnt[i] = 0;
        if (tid == 0) S.next_packet = 0;
        __syncthreads();
        const int64_t gid0 = (sg.ray_begin >> 2) + (c - sg.chunk_begin) * (int64_t)kChunkDraws;
        const uint32_t sid = (p.compat & RF_COMPAT_STREAMS) ? 0u : (p.scene_id + (uint32_t)sg.scene);
        const HitRec *gtab = p.tab + si.prim_off;
        unsigned long long *grow = p.hits + si.hits_off + (int64_t)cur_emitter * si.n;

        if (si.n <= kBruteMax) {  // block-uniform: too few surfaces for culling to pay
            // every thread traces its own rays against all surfaces in index order
            const int skip = self_skip(S.emit, cur_emitter);  // block-uniform
            uint32_t nv_warp = 0;
#pragma unroll 1
            for (int g = 0; g < kBatchDraws; ++g) {
                const int d = g * kBatchThreads + tid;
                const int64_t gid = gid0 + d;
                const bool any = gid * 4 + 3 >= sg.ray_begin && gid * 4 < sg.ray_end;
                const uint4 u = any ? stream_bits(p.compat, p.key1, sid, sg.emitter, gid) : make_uint4(0u, 0u, 0u, 0u);
                const float uf[4] = {u01(u.x), u01(u.y), u01(u.z), u01(u.w)};
#pragma unroll
                for (int v = 0; v < 4; ++v) {
                    const int64_t rid = gid * 4 + v;
                    const bool valid = rid >= sg.ray_begin && rid < sg.ray_end;
                    int bi = -1;
                    if (valid && BV) {
                        float r[4];
#pragma unroll
                        for (int i = 0; i < 4; ++i) r[i] = uf[(i + v + 1) & 3];
                        const Ray<float> ray = emit_mixed(S.emit, S.frame, r);
                        auto find = [&](int lo, int hi) {  // every child of [lo, hi), index order
                            float tr = MFast::inf();
                            int br = -1;
                            bool dr = false;
                            for (int j = lo; j < hi; ++j) {
                                if (j == skip) continue;
                                const HitRec h = S.tab[j];
                                const int type = __float_as_int(h.aux.x);
                                bool defer = false;
                                int idx;
                                const float t = test_mixed<STK>(type, h, j, S.tab, true, ray, eps, sc, defer, idx);
                                if (t < tr) { tr = t; br = idx; }
                                dr |= defer;
                                if (STK && is_stack(type)) j = stack_end(h, j) - 1;
                            }
                            return resolve_brute<STK>(br, dr, lo, hi, true, S.tab, gtab, ray, eps, sc, skip, nref);
                        };
                        bi = bv_select<false>(S.bvtab, S.bvinfo, S.bvbs, p.nbv, ray, eps, sc,
                                              (p.compat & RF_COMPAT_BV_STALE) != 0, find);
                    } else if (valid) {
                        float r[4];
#pragma unroll
                        for (int i = 0; i < 4; ++i) r[i] = uf[(i + v + 1) & 3];
                        const Ray<float> ray = emit_mixed(S.emit, S.frame, r);
                        float tb = MFast::inf();
                        bool dany = false;
#pragma unroll 1
                        for (int j = 0; j < si.n; ++j) {
                            if (j == skip) continue;  // uniform: every thread's emitter
                            const HitRec h = RESIDENT ? S.tab[j] : load_rec(gtab, j);
                            const int type = __float_as_int(h.aux.x);
                            bool defer = false;
                            int idx;
                            const float t = test_mixed<STK>(type, h, j, RESIDENT ? S.tab : gtab, RESIDENT, ray, eps, sc,
                                                            defer, idx);
                            if (t < tb) { tb = t; bi = idx; }
                            dany |= defer;
                            if (STK && is_stack(type)) j = stack_end(h, j) - 1;
                        }
                        bi = resolve_brute<STK>(bi, dany, 0, si.n, RESIDENT, S.tab, gtab, ray, eps, sc, skip, nref);
                    }
                    // all 32 lanes reach the warp-wide calls below
                    if (COUNT) nv_warp += __popc(__ballot_sync(0xffffffffu, valid));
                    if (REC) {
                        if (valid) p.rec[gid0 * 4 + 4 * d + v - p.rec_base] = bi;
                    } else if (hist_on) {
                        warp_tally(S.hist, bi);
                    } else {
                        warp_tally_global(grow, bi);
                    }
                }
            }
            if (COUNT) {
                if (lane == 0 && nv_warp)
                    for (int j = 0; j < si.n; ++j) {
                        if (j == skip) continue;
                        const HitRec h = RESIDENT ? S.tab[j] : load_rec(gtab, j);
                        const int type = __float_as_int(h.aux.x);
                        if (STK && is_stack(type)) {
                            S.wcount[warp][type == kStackType ? RF_CYLINDER : RF_ANNULUS] += nv_warp;
                            j = stack_end(h, j) - 1;
                        } else if ((unsigned)type < 6u) {
                            S.wcount[warp][type] += nv_warp;
                        }
                    }
                fold_counts();
            }
            __syncthreads();
            continue;
        }

        // 1. uniforms and sort keys (draw d = g*blockDim + tid, ray l = 4d + v);
        // keys go to perm[l] until the sort
#pragma unroll 1
        for (int g = 0; g < kBatchDraws; ++g) {
            const int d = g * kBatchThreads + tid;
            const int64_t gid = gid0 + d;
            uint2 kk = make_uint2(kCells | (kCells << 16), kCells | (kCells << 16));  // no valid ray
            if (gid * 4 + 3 >= sg.ray_begin && gid * 4 < sg.ray_end) {
                const uint4 u = stream_bits(p.compat, p.key1, sid, sg.emitter, gid);
                pack_uniforms(u, S.unif[0][d], S.unif[1][d], S.unif[2][d]);
                const float uf[4] = {u01(u.x), u01(u.y), u01(u.z), u01(u.w)};
                int key4[4];
#pragma unroll
                for (int v = 0; v < 4; ++v) {
                    float r[4];
#pragma unroll
                    for (int i = 0; i < 4; ++i) r[i] = uf[(i + v + 1) & 3];
                    const Ray<float> ray = emit_mixed(S.emit, S.frame, r);  // the origin is dead code here
                    const int64_t rid = gid * 4 + v;
                    const bool valid = rid >= sg.ray_begin && rid < sg.ray_end;
                    key4[v] = valid ? ray_key(ray, r) : kCells;
                    if (valid) atomicAdd(&S.cnt[key4[v]], 1);
                }
                kk = make_uint2((uint32_t)key4[0] | ((uint32_t)key4[1] << 16),
                                (uint32_t)key4[2] | ((uint32_t)key4[3] << 16));
            }
            *reinterpret_cast<uint2 *>(&S.perm[4 * d]) = kk;
        }
        __syncthreads();
        uint2 mykeys[kBatchDraws];
#pragma unroll
        for (int g = 0; g < kBatchDraws; ++g)
            mykeys[g] = *reinterpret_cast<const uint2 *>(&S.perm[4 * (g * kBatchThreads + tid)]);
        // 2. counting sort: block-wide exclusive scan of the bucket sizes (four
        // consecutive buckets per thread), then each ray claims a slot of its
        // bucket (in any order: a ray's result does not depend on its packet)
        {
            const int4 c4 = *reinterpret_cast<const int4 *>(&S.cnt[4 * tid]);
            const int sum = c4.x + c4.y + c4.z + c4.w;
            int incl = sum;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += t;
            }
            if (lane == 31) S.wsum[warp] = incl;
            __syncthreads();
            if (warp == 0) {
                const int x = S.wsum[lane];
                int xi = x;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int t = __shfl_up_sync(0xffffffffu, xi, o);
                    if (lane >= o) xi += t;
                }
                S.wsum[lane] = xi - x;
                if (lane == 31) S.n_valid = xi;
            }
            __syncthreads();
            const int run = S.wsum[warp] + incl - sum;
            *reinterpret_cast<int4 *>(&S.cnt[4 * tid]) =
                make_int4(run, run + c4.x, run + c4.x + c4.y, run + c4.x + c4.y + c4.z);
        }
        __syncthreads();
#pragma unroll
        for (int g = 0; g < kBatchDraws; ++g) {
            const int d = g * kBatchThreads + tid;
#pragma unroll
            for (int v = 0; v < 4; ++v) {
                const uint32_t w = (v < 2) ? mykeys[g].x : mykeys[g].y;
                const int key = (int)((w >> (16 * (v & 1))) & 0xffffu);
                if (key < kCells) S.perm[atomicAdd(&S.cnt[key], 1)] = (uint16_t)(4 * d + v);
            }
        }
        __syncthreads();
        const int n_valid = S.n_valid;

        // 3-5. warps take packets of 32 sorted rays; candidates are the union of
        // the rays' cell masks (or the surfaces the packet's bounds can reach);
        // each candidate gets the lanes' own gates and, if any lane passes, the
        // full test (index order, so ties go to the lower index as in
        // RayFactorGPU.cl:463-467); first hits are tallied at once
        constexpr bool resident = RESIDENT;
        const float4 *gbs = p.bsph + si.prim_off;
        const int n_packets = (n_valid + 31) >> 5;
        const int nwords_all = (si.n + 31) >> 5;
        for (;;) {
            int k = 0;
            if (lane == 0) k = atomicAdd(&S.next_packet, 1);
            k = __shfl_sync(0xffffffffu, k, 0);
            if (k >= n_packets) break;  // warp-uniform
            const int pos = k * 32 + lane;
            const bool valid = pos < n_valid;
            const int nvalid = COUNT ? __popc(__ballot_sync(0xffffffffu, valid)) : 0;  // every lane
            int bi = -1;
            {
                // re-emit the lane's ray (an invalid lane traces the packet's first ray)
                const int l = S.perm[valid ? pos : k * 32];
                const int d = l >> 2, v = l & 3;
                float uf[4], r[4];
                unpack_uniforms(S.unif[0][d], S.unif[1][d], S.unif[2][d], uf);
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const int q = (i + v + 1) & 3;
                    r[i] = q == 0 ? uf[0] : (q == 1 ? uf[1] : (q == 2 ? uf[2] : uf[3]));
                }
                const Ray<float> ray = emit_mixed(S.emit, S.frame, r);
                const float idd = MFast::rcp(ray.cx * ray.cx + ray.cy * ray.cy + ray.cz * ray.cz);
                const uint32_t *mcell = mrow ? mrow + (int64_t)ray_key(ray, r) * nwords_all : nullptr;
                if constexpr (BV) {
                    // runBVGPU: the nearest child in each bounding surface's range with the
                    // packet's culled candidate loop restricted to the range, then the walk
                    const int skip = self_skip(S.emit, cur_emitter);
                    if (COUNT && lane == 0) S.wcount[warp][7] += 1;
                    unsigned cmask = 0u;  // without masks: lane w holds candidate word w (n <= kBatchTile)
                    if (!mcell) {
                        const Packet pk = packet_bounds(ray, idd);
#pragma unroll 1
                        for (int w = 0; w < nwords_all; ++w) {
                            const int js = (w << 5) + lane;
                            const bool cand = js < si.n && packet_may_hit(pk, S.bs[js]);
                            const unsigned cm = __ballot_sync(0xffffffffu, cand);
                            if (lane == w) cmask = cm;
                        }
                    }
                    auto find = [&](int lo, int hi) {  // warp-wide: every lane, same lo and hi
                        float tr = MFast::inf();
                        int br = -1, dr = -1, nd = 0, skip_to = lo;
#pragma unroll 1
                        for (int w = lo >> 5; lo < hi && w <= (hi - 1) >> 5; ++w) {
                            const int jw = w << 5;
                            unsigned cm = mcell ? __reduce_or_sync(0xffffffffu, __ldg(mcell + w))
                                                : __shfl_sync(0xffffffffu, cmask, w);
                            cm &= keep_from((STK ? skip_to : lo) - jw);  // lo, and stacks tested in an earlier word
                            if (hi < jw + 32) cm &= (1u << (hi - jw)) - 1u;
                            if (skip >= jw && skip < jw + 32) cm &= ~(1u << (skip - jw));
                            while (cm) {
                                const int j = jw + __ffs(cm) - 1;
                                cm &= cm - 1;
                                if (COUNT && lane == 0) S.wcount[warp][6] += 1;  // candidates checked
                                if (!__any_sync(0xffffffffu, ray_may_hit(ray, idd, S.bs[j]))) continue;
                                const HitRec h = S.tab[j];
                                const int type = __float_as_int(h.aux.x);
                                if (COUNT) tcount += lane == stat_type(type) ? nvalid : 0;
                                bool defer = false;
                                int idx = j;
                                unsigned nb = 0u;
                                const float t = STK ? hit_hot(type, h, j, S.tab, true, ray, eps, sc, defer, idx, jw, cm,
                                                              skip_to, hi, nb)
                                                    : hit_mixed(type, h, ray, eps, sc, defer);
                                if (t < tr) { tr = t; br = idx; }
                                nd += defer;
                                dr = defer ? j : dr;
                            }
                        }
                        // as below: nearest among the children the lane's own gate admits
                        bool again = valid && nd > 1;
                        if (valid && nd == 1) {
                            int dq;
                            const float t = test_f64<STK>(S.tab[dr], dr, ray, eps, sc, dq);
                            if (t < tr || (t == tr && br >= 0 && dq < br)) { tr = t; br = dq; }
                            ++nref;
                            again = !own_gate(mcell, dr, ray, idd, S.bs[dr]);
                        }
                        if (valid && !again && br >= 0) again = !own_gate(mcell, br, ray, idd, S.bs[br]);
                        if (again) {
                            br = retrace_f64<STK>(lo, hi, true, S.tab, gtab, S.bs, gbs, mcell, true, ray, idd, eps, sc, skip,
                                             nref);
                        }
                        return br;
                    };
                    bi = bv_select<true>(S.bvtab, S.bvinfo, S.bvbs, p.nbv, ray, eps, sc, (p.compat & RF_COMPAT_BV_STALE) != 0,
                                         find);
                } else {
                    float tb = MFast::inf();
                    int dj = -1, ndef = 0;  // deferred FP64 tests of this lane: the last one, and how many
                    if (COUNT && lane == 0) S.wcount[warp][7] += 1;
                    // surfaces in blocks of 1024 (one block when the scene has masks)
                    int skip_to = 0;  // members of a stack already tested are not candidates
#pragma unroll 1
                    for (int j0 = 0; j0 < si.n; j0 += 1024) {
                        const int nwords = min(32, (si.n - j0 + 31) >> 5);
                        unsigned cmask = 0u;  // without masks: lane w holds candidate word w
                        if (!mcell) {  // block-uniform
                            const Packet pk = packet_bounds(ray, idd);
                            const int self = self_skip(S.emit, cur_emitter);  // (masks leave it out already)
#pragma unroll 1
                            for (int w = 0; w < nwords; ++w) {
                                const int js = j0 + (w << 5) + lane;
                                bool cand = false;
                                if (js < si.n && js != self)
                                    cand = packet_may_hit(pk, resident ? S.bs[js] : __ldg(gbs + js));
                                const unsigned cm = __ballot_sync(0xffffffffu, cand);
                                if (lane == w) cmask = cm;
                            }
                        }
#pragma unroll 1
                        for (int w = 0; w < nwords; ++w) {
                            const int jw = j0 + (w << 5);
                            const unsigned cm0 = mcell ? __reduce_or_sync(0xffffffffu, __ldg(mcell + (jw >> 5)))
                                                       : __shfl_sync(0xffffffffu, cmask, w);  // block-uniform choice
                            unsigned cm = STK ? cm0 & keep_from(skip_to - jw) : cm0;
                            // two candidates per pass: their sphere checks are independent
                            // chains (latency hidden); tests still run in index order
                            while (cm) {  // cm is the same in every lane
                                const int ba_ = __ffs(cm) - 1;
                                cm &= cm - 1;
                                const int bb_ = cm ? __ffs(cm) - 1 : -1;
                                cm &= cm - 1;  // 0 stays 0
                                const int ja = jw + ba_, jb = jw + (bb_ >= 0 ? bb_ : ba_);
                                if (COUNT && lane == 0) S.wcount[warp][6] += bb_ >= 0 ? 2 : 1;  // candidates checked
                                const float4 sa = resident ? S.bs[ja] : __ldg(gbs + ja);
                                const float4 sb = resident ? S.bs[jb] : __ldg(gbs + jb);
                                const bool ma = ray_may_hit(ray, idd, sa);
                                const bool mb = bb_ >= 0 && ray_may_hit(ray, idd, sb);
                                const unsigned va = __ballot_sync(0xffffffffu, ma);
                                unsigned vb = __ballot_sync(0xffffffffu, mb);
#pragma unroll
                                for (int q = 0; q < 2; ++q) {
                                    if (!(q ? vb : va)) continue;  // warp-uniform
                                    const int j = q ? jb : ja;
                                    const HitRec h = resident ? S.tab[j] : load_rec(gtab, j);
                                    const int type = __float_as_int(h.aux.x);
                                    if (COUNT) tcount += lane == stat_type(type) ? nvalid : 0;
                                    bool defer = false;
                                    int idx = j;
                                    const float t = STK ? hit_hot(type, h, j, resident ? S.tab : gtab, resident, ray, eps,
                                                                  sc, defer, idx, jw, cm, skip_to, q ? INT_MAX : jb, vb)
                                                        : hit_mixed(type, h, ray, eps, sc, defer);
                                    if (t < tb) { tb = t; bi = idx; }
                                    ndef += defer;  // predicated, no branch
                                    dj = defer ? j : dj;
                                }
                            }
                        }
                    }
                    // The lane's result must be its nearest hit among the surfaces its own
                    // gate admits (the set its cell mask and sphere check select), which
                    // depends on the ray alone.  The loop above took the nearest over the
                    // packet's tested surfaces, a superset; when the winner passes the
                    // lane's gate it is also the nearest of the gated set (same index-order
                    // ties), otherwise -- or when the lane deferred more than one test --
                    // the lane re-traces over its gated set (cold).  A single deferred test
                    // is re-evaluated in FP64 (lower index wins a tie: it ran out of order).
                    bool retrace = valid && ndef > 1;
                    if (valid && ndef == 1) {
                        const HitRec hq = RESIDENT ? S.tab[dj] : load_rec(gtab, dj);
                        int dq;
                        const float t = test_f64<STK>(hq, dj, ray, eps, sc, dq);
                        if (t < tb || (t == tb && bi >= 0 && dq < bi)) { tb = t; bi = dq; }
                        ++nref;
                        retrace = !own_gate(mcell, dj, ray, idd, resident ? S.bs[dj] : __ldg(gbs + dj));
                    }
                    if (valid && !retrace && bi >= 0)
                        retrace = !own_gate(mcell, bi, ray, idd, resident ? S.bs[bi] : __ldg(gbs + bi));
                    if (retrace) {
                        bi = retrace_f64<STK>(0, si.n, RESIDENT, S.tab, gtab, S.bs, gbs, mcell, true, ray, idd, eps, sc,
                                         self_skip(S.emit, cur_emitter), nref);
                    }
                }
                if (REC && valid) p.rec[gid0 * 4 + l - p.rec_base] = bi;
            }
            if (!REC) {  // every lane: warp-aggregated tally
                if (hist_on) warp_tally(S.hist, valid ? bi : -1);
                else warp_tally_global(grow, valid ? bi : -1);
            }
        }
        fold_counts();
        __syncthreads();
    }
    if (!REC) flush();
    // FP64 re-evaluations of this thread
    int tot = nref;
#pragma unroll
    for (int o = 16; o; o >>= 1) tot += __shfl_xor_sync(0xffffffffu, tot, o);
    if (lane == 0 && tot && p.refined) atomicAdd(p.refined, (unsigned long long)tot);
    __syncthreads();
    if (COUNT && tid < 8 && p.work && S.work[tid]) atomicAdd(p.work + tid, S.work[tid]);
}

// ---------------------------------------------------------------------------
// Cell masks.  For a row (scene, emitter) and each of the kCells sort keys,
// bit j of the key's mask says whether any ray of that emitter whose key it is
// can reach surface j: origins in the parameter patch's ball (MaskInputs::patch,
// 16 per emitter), directions in the direction cell's cone (cone[2*cell],
// axis and cos in xyzw, sin in the next entry's x), surfaces covered by up to
// kChainMax spheres (chain; radius < 0 ends the list) and, for planar surfaces,
// the plane (plane.xyz unit normal, w = normal . point; w NaN: not planar), which
// no ray crosses when the whole ball lies on one side and every direction of the
// cone points away from it.  A ray from a ball B(c, rho) with a direction within
// theta of axis a comes within R of a point C only if angle(C - c, a) <=
// theta + asin((R + rho) / |C - c|).
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool cell_reaches(float4 ball, float4 axis_cos, float sin_t, float4 sph)
{
    const float vx = sph.x - ball.x, vy = sph.y - ball.y, vz = sph.z - ball.z;
    const float L2 = vx * vx + vy * vy + vz * vz;
    const float R = (sph.w + ball.w) * 1.0001f + 1e-5f * sqrtf(L2) + 1e-7f;
    if (L2 <= R * R) return true;
    const float va = vx * axis_cos.x + vy * axis_cos.y + vz * axis_cos.z;
    return va >= axis_cos.w * sqrtf(L2 - R * R) - sin_t * R;
}

__device__ __forceinline__ bool plane_separates(float4 ball, float4 axis_cos, float sin_t, float4 pl)
{
    if (!(pl.w == pl.w)) return false;  // not planar
    const float h = pl.x * ball.x + pl.y * ball.y + pl.z * ball.z - pl.w;
    const float na = pl.x * axis_cos.x + pl.y * axis_cos.y + pl.z * axis_cos.z;
    const float margin = ball.w * 1e-4f + 1e-6f * (fabsf(pl.w) + ball.w) + 1e-7f;
    if (h > ball.w + margin) return na >= sin_t + 1e-4f;     // every ray moves away on the + side
    if (h < -(ball.w + margin)) return -na >= sin_t + 1e-4f; // ... or on the - side
    return false;
}

static __global__ void __launch_bounds__(256) build_masks_kernel(MaskInputs in, uint32_t *out)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= in.total_words) return;
    int lo = 0, hi = in.nrows - 1;  // the row holding word t (rows sorted by off)
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (in.rows[mid].off <= t) lo = mid;
        else hi = mid - 1;
    }
    const MaskRow row = in.rows[lo];
    const SceneInfo si = in.scenes[row.scene];
    const int nwords = (si.n + 31) >> 5;
    const int64_t local = t - row.off;
    const int cell = (int)(local / nwords), w = (int)(local % nwords);
    const float4 ball = in.patch[(int64_t)(si.prim_off + row.emitter) * 16 + (cell & 15)];
    const float4 ac = in.cone[2 * (cell >> 4)];
    const float sin_t = in.cone[2 * (cell >> 4) + 1].x;
    uint32_t bits = 0u;
    for (int b = 0; b < 32; ++b) {
        const int j = 32 * w + b;
        if (j >= si.n) break;
        const int gj = si.prim_off + j;
        bool ok = false;
        for (int k = 0; k < kChainMax && !ok; ++k) {
            const float4 sph = in.chain[(int64_t)gj * kChainMax + k];
            if (sph.w < 0.0f) break;
            ok = cell_reaches(ball, ac, sin_t, sph);
        }
        const float4 pl = in.plane[gj];
        if (ok && plane_separates(ball, ac, sin_t, pl)) ok = false;
        if (j == row.emitter && pl.w == pl.w) ok = false;  // a planar emitter cannot hit itself (self_skip)
        bits |= (ok ? 1u : 0u) << b;
    }
    out[t] = bits;
}

}  // namespace rf
