"""GB300-native (sm_103a) implementation of sDEM's per-step particle hot path.

Modules:
  capi      ctypes binding of libsdem_gpu.so (include/sdem_gpu.h) + DEMSystem handle
  props     material tables (InitPrtclProperty / clc_BnryPrtcl_Prop restated)
  geometry  plane walls (G_add_PlaneWall restated)
  beds      seeded synthetic beds (the workloads)
  restart   reader/writer of the reference's restart file layout
  settle    gravity settling of a placed bed by the GPU path (the settled 1M bed)
  build     nvcc recipe of the native library
"""
from . import beds, geometry, props  # noqa: F401

__all__ = ["beds", "geometry", "props", "capi", "build", "restart", "settle"]


def __getattr__(name):
    if name in ("capi", "build", "restart", "settle"):
        import importlib
        return importlib.import_module(f".{name}", __name__)
    raise AttributeError(name)
