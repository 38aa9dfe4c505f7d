"""imd_gb300 -- GB300-native replacement of IMD's force, neighbour-list,
NVE and CG hot path: hand-written sm_103a CUDA kernels behind a C-ABI
(include/imdgpu.h, libimdgpu.so) with a thin Python host layer."""
from .api import (EAM2, FP64, MIXED, PAIR, GpuSystem, IMDGPUError,  # noqa: F401
                  lib, system_from_tables)

__version__ = "1.0"
