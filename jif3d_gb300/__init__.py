"""GB300-native implementation of jif3D's gravity / FTG / magnetic prism path.

``capi``    -- ctypes binding of the C ABI (include/jif3d_gb300.h)
``gravmag`` -- the jif3D-shaped host layer (models, data, implementations,
               calculators, transforms)
``build``   -- in-tree nvcc build of libjif3d_gb300.so for sm_103a
"""
from . import build  # noqa: F401

__all__ = ["build", "capi", "gravmag"]


def __getattr__(name):
    if name in ("capi", "gravmag"):
        import importlib
        return importlib.import_module(f".{name}", __name__)
    raise AttributeError(name)
