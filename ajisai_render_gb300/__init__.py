"""ajisai_render_gb300: GB300-native wavefront path tracer for Ajisai's
PT-MIS path over a PLOC BVH.  The compute runs in libajisai_gpu.so (hand
written sm_103a CUDA behind the C ABI of include/ajisai_gpu.h); this package
holds the host-side mirror of the reference's interface and the scene
descriptions."""
from . import scenes  # noqa: F401
from .api import (AggregateOptions, Context, CreateDefaultScene,  # noqa: F401
                  CreatePLOCAggregate, CreatePTRenderer, Film, GpuScene,
                  PTRenderer, PTRendererArgs)
