"""GB300-native state-vector engine behind qibojit's backend API.

``MetaBackend.load("gb300")`` (the new platform next to qibojit's
``PLATFORMS = ("numba", "cupy", "cuquantum")``, src/qibojit/backends/__init__.py:8)
returns a :class:`GB300Backend` whose gate application, collapse, probabilities and
sampling run as hand-written sm_103a CUDA kernels in ``libqibojit_gb300.so``.
"""
from __future__ import annotations

__version__ = "0.1.0"

PLATFORMS = ("gb300",)

_default = None


class MetaBackend:
    """Loads the platforms this package provides (backends/__init__.py:11-46)."""

    @staticmethod
    def load(platform: str = None, **kwargs):
        if platform in (None, "gb300"):
            from .backend import GB300Backend

            return GB300Backend(**kwargs)
        raise ValueError(f"Unknown platform {platform}; available: {PLATFORMS}")

    def list_available(self) -> dict:
        out = {}
        for platform in PLATFORMS:
            try:
                MetaBackend.load(platform=platform)
                out[platform] = True
            except Exception:
                out[platform] = False
        return out


def get_backend():
    global _default
    if _default is None:
        _default = MetaBackend.load("gb300")
    return _default


def set_backend(backend) -> None:
    global _default
    _default = backend
