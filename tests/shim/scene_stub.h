// scene_stub.h -- test stand-in for the reference's Scene class
// (RayFactorCL/Scene.h:21-32) where the reference checkout is absent: the same
// public members, filled from a table dump that the reference's own
// Scene::readScene produced (tests/golden/scenes/*.bin, "RFSC" format written by
// oracle/ref_tools/ref_scene_dump.cpp), so the shim sees exactly the tables the
// reference host would hand to runCL_GPURNG.
#pragma once
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

struct Primitive {  // RayfactorConstants.h:38-45
    float m[12];
    float invm[12];
    int32_t type;
    int32_t rayDensity;
    float util1;
    float util2;
};

struct BoundingVolume {  // RayfactorConstants.h:48-56
    float invm[12];
    int32_t type;
    int32_t settings;
    int32_t objStartIndex;
    int32_t objEndIndex;
    float util1;
    float util2;
};

class Scene {
public:
    float globalRayDensity = 0.0f;
    bool useBoundingVolumes = false;
    std::vector<Primitive> primitives;
    std::vector<BoundingVolume> boundingVolumes;

    void readScene(const char *path)
    {
        FILE *f = std::fopen(path, "rb");
        if (!f) return;
        char magic[4];
        int32_t np = 0, nb = 0, ubv = 0;
        if (std::fread(magic, 1, 4, f) == 4 && std::memcmp(magic, "RFSC", 4) == 0 &&
            std::fread(&np, 4, 1, f) == 1 && std::fread(&nb, 4, 1, f) == 1 &&
            std::fread(&globalRayDensity, 4, 1, f) == 1 && std::fread(&ubv, 4, 1, f) == 1 && np >= 0 && nb >= 0) {
            useBoundingVolumes = ubv != 0;
            primitives.resize((size_t)np);
            boundingVolumes.resize((size_t)nb);
            if (np && std::fread(primitives.data(), sizeof(Primitive), (size_t)np, f) != (size_t)np) primitives.clear();
            if (nb && std::fread(boundingVolumes.data(), sizeof(BoundingVolume), (size_t)nb, f) != (size_t)nb)
                boundingVolumes.clear();
        }
        std::fclose(f);
    }
};
