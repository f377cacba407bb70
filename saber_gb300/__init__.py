"""saber_gb300 — GB300-native seed-and-extend scoring path of SABER.

The compute runs in libsaber_gb300.so (hand-written sm_103a kernels behind a
C ABI, include/saber_gpu.h); this package is its host-side binding plus the
synthetic workload generators.  Importing it does not touch the GPU.
"""
from .gpu import (JOB_DTYPE, CudaBackend, Device, SaberGpuError, band_cells, load_library,
                  score_banded_many)
from .scoring import ALPHABET, encode_protein, matrix

__all__ = ["JOB_DTYPE", "CudaBackend", "Device", "SaberGpuError", "band_cells", "load_library",
           "score_banded_many", "ALPHABET", "encode_protein", "matrix"]
