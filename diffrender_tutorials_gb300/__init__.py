"""GB300-native differentiable mesh renderer (hot path of FROL256/diffrender_tutorials).

The compute path is libdrgb.so (CUDA kernels for sm_103a behind the C ABI in
include/drgb.h); this package holds the build script, the ctypes binding and
a Python mirror of the reference's IDiffRender / IOptimizer interfaces.
"""
from .scene import (CamInfo, Scene, Texture, TransformR, TriangleMesh, displace_radially, make_cube, make_icosphere,  # noqa: F401
                    make_uv_sphere, perturb_vertices, ring_cameras)
from .api import (SHADING_MODEL, CreateSimpleOptimizer, DiffRenderSettings, DMesh, DScene, IDiffRender,  # noqa: F401
                  IOptimizer, MakeDifferentialRenderer, ModelParams, OptimizerParameters, kernel_launches,
                  BatchOptimizer, OptimizationServer, estimate_job_bytes)
from . import io  # noqa: F401,E402  (mesh and image files)
