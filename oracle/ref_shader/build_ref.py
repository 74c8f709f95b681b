"""ORACLE — test infrastructure only. Recipe that compiles the reference's DDGI shaders as FP64 C++
(filled in below); on machines without the reference sources it does nothing."""
from __future__ import annotations

from pathlib import Path

REFERENCE = Path("/root/reference")


def build_if_available() -> Path | None:
    """Builds oracle/_ref/libddgi_refshader.so when the reference sources are present; returns its path
    or None."""
    if not (REFERENCE / "assets" / "shaders").is_dir():
        return None
    return None
