"""craystal_gb300 -- GB300-native (sm_103a) path-tracing hot path of CRaystal.

The public API mirrors the reference's Scene / Camera / Sensor /
PathTraceIntegrator classes; all work runs in libcraystal_gb300.so through
its C ABI (include/craystal_c.h).
"""
from ._lib import CrayError, HIT_DTYPE, MATERIAL_DTYPE, MESH_DTYPE, RAY_DTYPE, CR_MISS, LIB_PATH, load  # noqa: F401
from .api import (CachedPathTraceIntegrator, Camera, MaterialData, MaterialFlags, MaterialType, MeshData,  # noqa: F401
                  PathTraceIntegrator, RadianceCache, BatchRenderer,
                  Scene, SceneData, Sensor, flatten_scene, kernel_launch_count, version)
