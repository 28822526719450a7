"""GB300 (sm_103a) Monte Carlo view-factor tracer: a drop-in for the tracing
path of RayFactorCL (RayFactorCL/RayFactorGPU.cl and the launch logic of
RayFactorCL/main.cpp) behind the C ABI of include/rayfactor_gb300.h."""
from .scene import (ANNULUS, BV_DTYPE, CYLINDER, DISC, FRUSTUM, NONE, PRIM_DTYPE, RECTANGLE,  # noqa: F401
                    SPHERE, Scene, parse_scene_xml, read_scene)

__all__ = ["Scene", "read_scene", "parse_scene_xml", "PRIM_DTYPE", "BV_DTYPE", "Tracer",
           "run_cl_gpurng", "ray_budgets", "write_output_txt", "build"]


def build(force: bool = False):
    """Compile the CUDA library in tree (sm_103a)."""
    from .buildlib import build as _b
    return _b(force=force)


def __getattr__(name):
    if name in ("Tracer", "run_cl_gpurng", "ray_budgets", "write_output_txt"):
        from . import tracer
        return getattr(tracer, name)
    raise AttributeError(name)
