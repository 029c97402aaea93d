"""GB300 renderer core for Dayflower's path tracer: Python host side.

RendererKernel mirrors the reference's AbstractRendererKernel/GPURendererKernel method set and
drives libdfpt.so through its C-ABI (include/dfpt.h). There is no CPU fallback.
"""
from .scene import CompiledScene, SceneBuilder, SkyState  # noqa: F401
from .kernel import RendererKernel  # noqa: F401
