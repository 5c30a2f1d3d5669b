"""GB300-native gravity force evaluation for ChaNGa-style tree codes.

The product is the CUDA library behind include/HostCUDA.h,
include/EwaldCUDA.h and include/changa_gb300.h; this package holds its
sources (csrc/), the host-side tree/walk that produces its inputs (host/,
tree.py), seeded workloads (ics.py) and Python wrappers (gravity.py).
"""
__all__ = ["ics", "tree", "gravity", "build"]
