// shim_main.cpp -- test program for include/rayfactor_gb300_shim.hpp: the
// reference's main() (RayFactorCL/main.cpp:275-284) with runCL_GPURNG replaced
// by runCUDA_GPURNG.  Built twice by the tests:
//   * with the reference's own Scene.h / Scene.cpp / TinyXML-2 / affine code
//     (CPU test, where the reference checkout exists): argv[1] is a scene XML;
//   * with -DRF_SHIM_SCENE_STUB and scene_stub.h (GPU test): argv[1] is a table
//     dump written by the reference's loader (tests/golden/scenes/*.bin).
// argv[2] (optional): compat bits, default RF_COMPAT_ALL.  Writes output.txt in
// the working directory like the reference.
#include <cstdlib>

#ifdef RF_SHIM_SCENE_STUB
#include "scene_stub.h"
#else
#include "Scene.h"
#endif
#include "rayfactor_gb300_shim.hpp"

int main(int argc, const char *argv[])
{
    Scene scene;
    const char *xmlpath = argc > 1 ? argv[1] : "input.xml";
    scene.readScene(xmlpath);
    const uint32_t compat = argc > 2 ? (uint32_t)std::strtoul(argv[2], nullptr, 0) : RF_COMPAT_ALL;
    return runCUDA_GPURNG((int)scene.globalRayDensity, scene, compat);
}
