/*
 * rayfactor_gb300_shim.hpp -- drop-in replacement for RayFactorCL's
 * runCL_GPURNG(int n_samples, Scene &scene) (RayFactorCL/main.cpp:54-272) on top
 * of the C ABI in rayfactor_gb300.h.
 *
 * Header-only and a template over the caller's Scene class, so it needs none of
 * the reference's headers: any class with the members the reference's Scene
 * has (RayFactorCL/Scene.h:21-25) works --
 *     float globalRayDensity;  bool useBoundingVolumes;
 *     std::vector<Primitive> primitives;  std::vector<BoundingVolume> boundingVolumes;
 * with Primitive / BoundingVolume laid out as in RayFactorCL/RayfactorConstants.h:38-56
 * (checked at compile time against rf_primitive / rf_bounding_volume).
 *
 * In the reference's main.cpp, include this header after Scene.h and call
 *     runCUDA_GPURNG((int)scene.globalRayDensity, scene);
 * in place of runCL_GPURNG(scene.globalRayDensity, scene) (main.cpp:275-284);
 * link with -lrayfactor_gb300.
 *
 * Same budgets (main.cpp:172-173), same kernel choice by useBoundingVolumes
 * (main.cpp:68-75), same normalisation (main.cpp:178, 241-249) and the same
 * output.txt format (main.cpp:236-249).  compat selects the reference's
 * behaviours (RF_COMPAT_ALL: identical streams, budgets and quirks; 0: fixed).
 * Returns 0 on success; on failure prints rf_last_error to stderr and returns 1
 * instead of exiting (the reference's CHECK macros exit, util_opencl.h:123-131).
 */
#ifndef RAYFACTOR_GB300_SHIM_HPP
#define RAYFACTOR_GB300_SHIM_HPP

#include <cstdio>
#include <vector>

#include "rayfactor_gb300.h"

template <class SceneT>
int runCUDA_GPURNG(int n_samples, SceneT &scene, uint32_t compat = RF_COMPAT_ALL,
                   const char *output_path = "output.txt")
{
    typedef typename decltype(scene.primitives)::value_type PrimT;
    typedef typename decltype(scene.boundingVolumes)::value_type BvT;
    static_assert(sizeof(PrimT) == sizeof(rf_primitive), "Primitive layout (RayfactorConstants.h:38-45)");
    static_assert(sizeof(BvT) == sizeof(rf_bounding_volume), "BoundingVolume layout (RayfactorConstants.h:48-56)");

    rf_config cfg;
    rf_config_default(&cfg);
    cfg.compat = compat;
    rf_ctx *ctx = nullptr;
    rf_status s = rf_create(&ctx, &cfg);
    if (s != RF_OK) {
        std::fprintf(stderr, "rayfactor_gb300: %s\n", ctx ? rf_last_error(ctx) : rf_status_string(s));
        rf_destroy(ctx);
        return 1;
    }
    const int n = (int)scene.primitives.size();
    const int nbv = (int)scene.boundingVolumes.size();
    s = rf_set_scene(ctx, reinterpret_cast<const rf_primitive *>(scene.primitives.data()), n,
                     nbv ? reinterpret_cast<const rf_bounding_volume *>(scene.boundingVolumes.data()) : nullptr,
                     nbv);
    std::vector<double> F((size_t)n * (size_t)n);
    if (s == RF_OK) s = rf_run_gpurng(ctx, n_samples, scene.useBoundingVolumes ? 1 : 0, nullptr, nullptr, F.data());
    if (s == RF_OK) s = rf_write_output_txt(output_path, F.data(), n);
    if (s != RF_OK) std::fprintf(stderr, "rayfactor_gb300: %s\n", rf_last_error(ctx));
    rf_destroy(ctx);
    return s == RF_OK ? 0 : 1;
}

#endif
