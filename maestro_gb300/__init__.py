"""GB300-native (CUDA sm_103a) MAC projection for MAESTRO.

The product is the C-ABI library ``_lib/libmaestro_mac.so`` (declared in include/maestro_mac.h);
this package holds its CUDA sources (``csrc/``), the build step, the ctypes binding, the host-side
mirror of MAESTRO's ``macproject`` / ``mac_multigrid`` interface and the seeded synthetic inputs.
"""
from .build import build  # noqa: F401

__all__ = ["build"]
