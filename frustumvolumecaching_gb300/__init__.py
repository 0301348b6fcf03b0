"""GB300-native frustum-volume-caching NeRF renderer.

The compute path is libfvc.so (hand-written CUDA for sm_103a behind the C ABI
of include/fvc.h); this package holds its ctypes binding, the Python mirror of
the reference's renderer API, and the seeded synthetic-model generator.
"""
from .renderer import (BasicRenderer, Cache, CacheBasicRenderer, CachePerformanceRenderer, Gradients, LoaderData, NerfNetwork,  # noqa: F401
                       PerformanceRenderer, RenderBuffer, Renderer, camera_info, default_cache_settings, ingp_export,
                       load_data, raymarch_info, eval_cache_settings, change_sampling_rate, DENSITY, ALPHA, INTERMEDIATES,
                       DENSITY_INTERMEDIATES, ALPHA_INTERMEDIATES, LINEAR, SMOOTHSTEP, SMOOTHERSTEP, NEAREST)
