// ref_scene_dump.cpp -- test infrastructure.  Parses a scene XML with the
// reference's own loader (RayFactorCL/Scene.cpp:24-452 with TinyXML-2 and the
// affine code in RayFactorCL/Affine Transformation/) and writes the resulting
// tables in binary:
//   "RFSC" | int32 n_prims | int32 n_bvs | float globalRayDensity |
//   int32 useBoundingVolumes | n_prims x 112-byte Primitive | n_bvs x 72-byte BoundingVolume
// The reference leaves some fields uninitialised (Scene.h:25 useBoundingVolumes,
// Scene.cpp:107-110 settings, util1/util2 of discs and rectangles); operator new
// is replaced here by a zero-filling allocator so those read as 0 and the dump
// is deterministic.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include "Scene.h"

void *operator new(std::size_t n)
{
    void *p = std::calloc(1, n ? n : 1);
    if (!p) throw std::bad_alloc();
    return p;
}
void operator delete(void *p) noexcept { std::free(p); }
void operator delete(void *p, std::size_t) noexcept { std::free(p); }

int main(int argc, char **argv)
{
    if (argc != 3) {
        std::fprintf(stderr, "usage: %s scene.xml out.bin\n", argv[0]);
        return 2;
    }
    static_assert(sizeof(Primitive) == 112, "Primitive layout");
    static_assert(sizeof(BoundingVolume) == 72, "BoundingVolume layout");
    Scene *scene = new Scene();
    scene->readScene(argv[1]);
    FILE *f = std::fopen(argv[2], "wb");
    if (!f) return 1;
    int32_t np = (int32_t)scene->primitives.size(), nb = (int32_t)scene->boundingVolumes.size();
    float grd = scene->globalRayDensity;
    int32_t ubv = scene->useBoundingVolumes ? 1 : 0;
    std::fwrite("RFSC", 1, 4, f);
    std::fwrite(&np, 4, 1, f);
    std::fwrite(&nb, 4, 1, f);
    std::fwrite(&grd, 4, 1, f);
    std::fwrite(&ubv, 4, 1, f);
    if (np) std::fwrite(scene->primitives.data(), sizeof(Primitive), np, f);
    if (nb) std::fwrite(scene->boundingVolumes.data(), sizeof(BoundingVolume), nb, f);
    std::fclose(f);
    return 0;
}
