"""GB300-native wavefront path-tracing render core for Lighthouse 2 (CUDA sm_103a).

The compute path is the CUDA library libRenderCore_GB300.so (C ABI: include/lh2g.h; Lighthouse 2 plugin ABI:
include/lh2_core_api.h). This package holds its build recipe, a ctypes mirror of the plugin interface
(core.RenderCore) and the seeded scene generators used by the tests and the benchmark.
"""
from .core import RenderCore, CoreError, load_library, make_params, camera_r0  # noqa: F401
