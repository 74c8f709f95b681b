"""GB300-native DDGI probe-update engine: LBVH build, probe-ray traversal and hit shading, probe
convolution and probe translation as sm_103a CUDA behind the C ABI of include/ddgi.h."""
from . import _lib  # noqa: F401

__all__ = ["_lib"]
