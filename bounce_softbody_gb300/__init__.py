"""bounce_softbody_gb300: the implicit soft-body step of Bounce Softbody on GB300 (sm_103a).

The product is libb3g.so and its C ABI (include/b3g.h); this package holds the CUDA sources
(csrc/), the in-tree build recipe (build.py), the ctypes binding of the C ABI (b3g.py) and the
seeded workload generators (meshes.py).
"""
from . import meshes  # noqa: F401

__all__ = ["meshes", "b3g", "build"]
