"""GB300-native (sm_103a) re-implementation of SwiftShader's triangle draw hot
path behind a C-ABI shaped like sw::Renderer::draw.

Modules:
  abi       -- ctypes mirror of include/swgb.h
  build     -- in-tree nvcc build of libswgb.so
  renderer  -- Renderer (draw / draw_batch / synchronize), DeviceScene, DeviceBatch
  scenes    -- seeded synthetic workloads
"""
from . import abi, scenes  # noqa: F401

__all__ = ["abi", "scenes", "Renderer", "DeviceScene", "DeviceBatch"]


def __getattr__(name):
    if name in ("Renderer", "DeviceScene", "DeviceBatch"):
        from . import renderer
        return getattr(renderer, name)
    raise AttributeError(name)
