"""msplat_gb300 — a GB300-native (sm_103a) 3D Gaussian Splatting training engine
behind msplat's C API.

Layers:
  include/msplat_c_api.h   the reference's public C API (trainer, dataset, viewer)
  include/msplat_engine.h  the device-level step (msplat_train_step / msplat_render)
  msplat_gb300/csrc        CUDA kernels + C++ host, built into libmsplat_gb300.so
  msplat_gb300.engine      Python handle on the engine (tests, benchmarks)
"""
from . import synthetic  # noqa: F401

__all__ = ["synthetic", "build", "engine"]
