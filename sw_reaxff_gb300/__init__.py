"""GB300-native ReaxFF force step (bond orders, bonded terms, H-bonds,
vdW+Coulomb, QEq, NVE) behind the reaxgpu C ABI (include/reaxgpu.h).

Layout:
  csrc/        CUDA kernels (sm_103a) and the C-ABI host code
  api.py       ctypes binding of libreaxgpu.so
  lammps.py    host-side mirror of the LAMMPS plugin classes
  systems.py   seeded synthetic workloads
  build.py     in-tree nvcc build of libreaxgpu.so
"""
from .api import (DEFAULT_FFIELD, ENERGY_NAMES, ReaxError, ReaxGPU,  # noqa: F401
                  load_library)
