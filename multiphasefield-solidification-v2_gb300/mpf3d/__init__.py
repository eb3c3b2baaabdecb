"""mpf3d -- GB300-native (sm_103a) 3D multi-phase-field step.

Tiers
-----
* ``mpf3d.dense``: the reference's kernels on its dense arrays with its
  numerics (backs the drop-in module ``src/gpu_kernels_3d.py``).
* further tiers are added as modules of this package.

All compute runs in libmpf3d.so (hand-written CUDA for sm_103a, C ABI in
include/mpf3d.h).  There is no CPU fallback.
"""

from . import _lib  # noqa: F401
from .inputs import Physics  # noqa: F401

KMAX = 50
LIQ = 0
