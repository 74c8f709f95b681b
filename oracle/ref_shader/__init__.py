"""ORACLE — test infrastructure only. The reference's shader sources compiled as FP64 C++ (see build_ref)."""
from .build_ref import build_if_available  # noqa: F401
