"""spinifel_gb300: GB300-native (sm_103a) slicing, orientation matching and
3D NUFFT operators for Spinifel's M-TIP reconstruction.

Compute runs in libspinifel_gb300.so (hand-written CUDA, C ABI in
include/spinifel_gb300.h); this package is the host side that mirrors the
reference's Python call surface.
"""
from .settings import Settings, SpinifelSettings  # noqa: F401

__version__ = "0.1.0"
