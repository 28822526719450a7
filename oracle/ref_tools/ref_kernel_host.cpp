// ref_kernel_host.cpp -- test infrastructure.  Driver appended by
// oracle/build.py after cl_compat.h and the reference's own kernel source
// (RayFactorCL/RayFactorGPU.cl) in one g++ translation unit.  It runs the
// reference's runGPU (RayFactorGPU.cl:481-527) or runBVGPU (:530-626) one
// work-item at a time, as the OpenCL runtime would for global ids
// [gid_begin, gid_end) of one emitter, and returns the first-hit surface of
// each of the 4 sub-rays of every work-item (-1 = no hit), in the order ray
// 4*gid + v.  Built into oracle/_ref/librf_refkernel.so; tests load it through
// ctypes to pin the oracle's per-ray results to the reference kernel itself.
#include <cstdlib>
#include <vector>

extern "C" int rfr_trace_rays(const void *prims, int32_t n_objects, const void *bvs, int32_t n_bvs,
                              int32_t use_bv, int32_t emitter, int64_t gid_begin, int64_t gid_end,
                              int32_t *out)
{
    static_assert(sizeof(Primitive) == 112, "Primitive layout (RayfactorConstants.h:38-45)");
    static_assert(sizeof(BoundingVolume) == 72, "BoundingVolume layout (RayfactorConstants.h:48-56)");
    if (!prims || !out || n_objects <= 0 || emitter < 0 || emitter >= n_objects || gid_begin < 0 ||
        gid_end < gid_begin || gid_end > ((int64_t)1 << 31) || (use_bv && (!bvs || n_bvs <= 0)))
        return -1;
    std::vector<int> hits((size_t)n_objects * (size_t)n_objects, 0);
    g_rfcl.hits = hits.data();
    g_rfcl.n_objects = n_objects;
    g_rfcl.from = emitter;
    const Primitive *objects = static_cast<const Primitive *>(prims);
    const BoundingVolume *bv = static_cast<const BoundingVolume *>(bvs);
    for (int64_t gid = gid_begin; gid < gid_end; ++gid) {
        g_rfcl.gid = (size_t)gid;
        g_rfcl.base = out + 4 * (gid - gid_begin);
        g_rfcl.nslots = 0;
        if (use_bv)
            runBVGPU(emitter, n_objects, objects, nullptr, hits.data(), n_bvs, bv);
        else
            runGPU(emitter, n_objects, objects, nullptr, hits.data());
        if (g_rfcl.nslots != 4) return -2;  // every work-item forms exactly four sub-rays
    }
    return 0;
}
