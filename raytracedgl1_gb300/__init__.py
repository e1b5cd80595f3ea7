"""GB300-native A-SVGF denoise + luminance-histogram auto-exposure (the image-space hot path
of RayTracedGL1), behind the C ABI of include/rgdn.h."""
from . import _native  # noqa: F401

__all__ = ["_native"]
