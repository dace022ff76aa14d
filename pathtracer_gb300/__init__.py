"""GB300-native (sm_103a) spectral path tracer behind the C ABI of
phyastro/PathTracer's compute dispatch.

The product is native: libpt_cuda.so (CUDA kernels + C ABI, include/pt_cuda.h)
and libpt_host.so (headless scene/packing/offscreen host, include/pt_host.h).
This package builds them in-tree (``build.build()``) and binds them with
ctypes (``native``, ``renderer``).
"""
from .renderer import (  # noqa: F401
    Batch, Context, PathTracerError, Scene, Server, cie_analytic, export_rgb8, glsl_translate, jit_check,
    render_offscreen)

SCENES_DIR = __import__("os").path.join(__import__("os").path.dirname(__file__), "scenes")
