"""GB300-native (sm_103a) SPH substep engine with libclsph's sph_simulation API.

Modules:
  layout     byte layouts of particle / simulation_parameters / kernel terms
  settings   load_settings: property files and the derived parameter block
  gpu        ctypes binding of the C ABI (include/clsph_gpu.h)
  simulation Python mirror of sph_simulation / scene / houdini_file_saver
  workloads  seeded synthetic scenes of the benchmark shapes
  build      nvcc / g++ recipes for the native libraries
"""

from . import layout, settings  # noqa: F401

__all__ = ["layout", "settings"]
