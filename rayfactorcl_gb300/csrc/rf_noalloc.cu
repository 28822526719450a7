// rf_noalloc.cu -- rf_trace_mixed_noalloc: the batched mixed-precision tracer
// for one scene, callable by hosts that must not allocate device memory.
//
// Who needs it: a host application that has already reserved the GPU's memory
// in its own pool (a simulation coupling the view factors into its solver, a
// plugin inside a renderer or CFD code) cannot let a library cudaMalloc more;
// a cudaMalloc can also synchronise the device and stall the host's other
// streams, which a latency-bound loop cannot afford.  Such a caller passes its
// own buffers for inputs and outputs; everything else the kernel needs (the
// prepared surface tables, the segment plan and the work-queue counters) lives
// in one file-scope device array of RF_NOALLOC_SCRATCH_BYTES, which every GPU
// that loads this library holds until the process exits.
#include <cmath>
#include <cstring>
#include <mutex>

#include <cuda_runtime.h>

#include "rayfactor_gb300.h"
#include "rf_internal.h"

using namespace rf;

namespace {

constexpr int kMaxPrims = RF_NOALLOC_MAX_PRIMS;
// the call always launches the kernel variant that keeps the scene's tables in
// shared memory, which holds kBatchTile surfaces
static_assert(kMaxPrims <= kBatchTile, "RF_NOALLOC_MAX_PRIMS must fit the resident kernel's tables");
constexpr int kMaxDevices = 128;

// Layout of the scratch array.
constexpr size_t kOffCounters = 0;                                   // queue, refined, work[8]
constexpr size_t kOffScene = 256;                                    // one SceneInfo
constexpr size_t kOffSeg = 512;                                      // kMaxPrims segments
constexpr size_t kOffTab = kOffSeg + sizeof(Segment) * kMaxPrims;    // hit records
constexpr size_t kOffEmit = kOffTab + sizeof(HitRec) * kMaxPrims;    // emitter records
constexpr size_t kOffSph = kOffEmit + sizeof(rf_primitive) * kMaxPrims;  // bounding spheres
constexpr size_t kOffFrame = kOffSph + sizeof(float4) * kMaxPrims;      // planar emission frames
constexpr size_t kScratchUsed = kOffFrame + sizeof(float4) * kEmitFrameWords * kMaxPrims;
static_assert(kScratchUsed <= RF_NOALLOC_SCRATCH_BYTES, "scratch layout exceeds the stated size");
static_assert(kOffTab % 16 == 0 && kOffEmit % 16 == 0 && kOffSph % 16 == 0 && kOffFrame % 16 == 0,
              "16-byte alignment");

struct Counters {
    unsigned long long queue;
    unsigned long long refined;
    unsigned long long work[8];
};
static_assert(sizeof(Counters) <= kOffScene, "counters fit their slot");

__device__ __align__(256) unsigned char g_scratch[RF_NOALLOC_SCRATCH_BYTES];

// Device address of g_scratch per device, looked up once; in host code the
// symbol itself is only a host-side stand-in and must not be handed to a kernel.
std::mutex g_mu;
unsigned char *g_dev[kMaxDevices] = {};

// Host staging of the prepared tables (static storage, no heap); the mutex
// serialises callers on different host threads while they fill it.
rf_primitive h_emit[kMaxPrims];
HitRec h_tab[kMaxPrims];
float4 h_sph[kMaxPrims];
float4 h_frame[kMaxPrims * kEmitFrameWords];
Segment h_seg[kMaxPrims];

bool finite12(const float *v)
{
    for (int i = 0; i < 12; ++i)
        if (!std::isfinite(v[i])) return false;
    return true;
}

}  // namespace

extern "C" rf_status rf_trace_mixed_noalloc(const rf_primitive *prims, int32_t n, const int64_t *rays,
                                            uint32_t compat, uint32_t key1, float eps, uint64_t *hits_dev,
                                            void *stream)
{
    if (!prims || !rays || !hits_dev || n <= 0) return RF_ERR_INVALID_ARG;
    if (n > kMaxPrims) return RF_ERR_OVERFLOW;  // the scratch array holds RF_NOALLOC_MAX_PRIMS surfaces
    if (!std::isfinite(eps)) return RF_ERR_INVALID_ARG;
    for (int i = 0; i < n; ++i) {
        const rf_primitive &p = prims[i];
        if (p.type < 0 || p.type > RF_DISC || !finite12(p.m) || !finite12(p.invm)) return RF_ERR_BAD_SCENE;
        if ((p.type == RF_FRUSTUM || p.type == RF_ANNULUS) && !std::isfinite(p.util1)) return RF_ERR_BAD_SCENE;
        if (p.type != RF_DISC && p.type != RF_RECTANGLE && !std::isfinite(p.util2)) return RF_ERR_BAD_SCENE;
        if (rays[i] < 0) return RF_ERR_INVALID_ARG;
        if (rays[i] > (1ll << 46)) return RF_ERR_OVERFLOW;
        if ((compat & RF_COMPAT_STREAMS) && rays[i] > (4ll << 32)) return RF_ERR_OVERFLOW;
    }
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return RF_ERR_NO_DEVICE;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return RF_ERR_CUDA;
    cudaStream_t st = static_cast<cudaStream_t>(stream);

    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_dev[dev]) {  // first call on this device
        void *ptr = nullptr;
        if (cudaGetSymbolAddress(&ptr, g_scratch) != cudaSuccess || !ptr) return RF_ERR_CUDA;
        g_dev[dev] = static_cast<unsigned char *>(ptr);
    }
    unsigned char *base = g_dev[dev];

    float seps = eps;  // eps < 0: relative to the scene's size, like rf_trace
    const int nstacks = prepare_mixed_tables(prims, n, eps, h_emit, h_tab, h_sph, &seps);
    for (int i = 0; i < n; ++i) emit_frame(h_emit[i], h_frame + (size_t)i * kEmitFrameWords);
    int nseg = 0;
    int64_t chunks = 0;
    for (int e = 0; e < n; ++e) {
        if (rays[e] <= 0) continue;
        Segment sg;
        sg.emitter = e;
        sg.scene = 0;
        sg.ray_begin = 0;
        sg.ray_end = rays[e];
        sg.chunk_begin = chunks;
        h_seg[nseg++] = sg;
        const int64_t draws = (rays[e] + 3) >> 2;
        chunks += (draws + kBatchChunkDraws - 1) / kBatchChunkDraws;
    }
    SceneInfo si{};
    si.n = n;
    si.prim_off = 0;
    si.hits_off = 0;
    si.eps = seps;

    // copies from pageable host memory return once the source has been staged,
    // so the static host tables may be refilled by the next caller
    cudaError_t e = cudaMemsetAsync(hits_dev, 0, sizeof(uint64_t) * (size_t)n * n, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(base + kOffCounters, 0, sizeof(Counters), st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(base + kOffScene, &si, sizeof si, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && nseg)
        e = cudaMemcpyAsync(base + kOffSeg, h_seg, sizeof(Segment) * nseg, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(base + kOffTab, h_tab, sizeof(HitRec) * n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(base + kOffEmit, h_emit, sizeof(rf_primitive) * n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(base + kOffSph, h_sph, sizeof(float4) * n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(base + kOffFrame, h_frame, sizeof(float4) * kEmitFrameWords * n, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return RF_ERR_CUDA;
    if (chunks == 0) return RF_OK;

    Counters *cnt = reinterpret_cast<Counters *>(base + kOffCounters);
    TraceParams p{};
    p.tab = reinterpret_cast<const HitRec *>(base + kOffTab);
    p.emit = reinterpret_cast<const rf_primitive *>(base + kOffEmit);
    p.bsph = reinterpret_cast<const float4 *>(base + kOffSph);
    p.frame = reinterpret_cast<const float4 *>(base + kOffFrame);
    p.scenes = reinterpret_cast<const SceneInfo *>(base + kOffScene);
    p.seg = reinterpret_cast<const Segment *>(base + kOffSeg);
    p.hits = reinterpret_cast<unsigned long long *>(hits_dev);
    p.queue = &cnt->queue;
    p.refined = &cnt->refined;
    p.work = cnt->work;
    p.total_chunks = chunks;
    p.nseg = nseg;
    p.compat = compat;
    p.key1 = key1;
    p.scene_id = 0;
    p.eps = seps;
    int bps = batched_blocks_per_sm(false, true);
    if (bps <= 0) bps = 1;
    const int grid = (int)(chunks < (int64_t)sms * bps ? chunks : (int64_t)sms * bps);
    return launch_batched(p, false, true, false, nstacks > 0, grid, st) == cudaSuccess ? RF_OK : RF_ERR_CUDA;
}
