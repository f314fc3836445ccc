"""GB300-native KDTree hot path of NBodylib: sm_103a CUDA kernels behind a C ABI.

``KDTree`` mirrors the reference's ``NBody::KDTree`` methods; ``BatchedDensity`` drives
the batched many-trees path; ``synthetic`` generates the seeded workloads.
"""
from .kdtree import (DEVICE_PTRS, FINDNEAREST, FINDNEARESTPOS, FOF3D, FOF6D, FOFVEL, KEPAN,
                     KGAUSS, KSPH, KTH, PERIODIC_MIN_IMAGE, PERIODIC_REF, TPHS, TPHYS, TPROJ,
                     TVEL, BatchedDensity, KDTree)

__all__ = ["KDTree", "BatchedDensity", "TPHYS", "TPROJ", "TVEL", "TPHS", "KSPH", "KGAUSS", "KEPAN", "KTH",
           "FINDNEAREST", "FINDNEARESTPOS", "PERIODIC_REF", "PERIODIC_MIN_IMAGE", "FOF3D",
           "FOFVEL", "FOF6D", "DEVICE_PTRS"]
