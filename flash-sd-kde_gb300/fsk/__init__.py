"""fsk - GB300-native kernels behind the Flash-SD-KDE drop-in API.

``fsk.ops`` wraps the C ABI of libfsk.so (include/fsk.h); ``fsk.workloads``
generates the seeded synthetic benchmark inputs; ``fsk.surrogate`` holds the
learned MLP surrogate.
"""
from . import _lib  # noqa: F401

__all__ = ["ops", "workloads"]
