"""Overlay for the reference's ``src`` package.

Only ``src/gpu_kernels_3d.py`` is replaced.  When ``MPF3D_REFERENCE_SRC``
names the reference's ``src`` directory, its other modules
(``orientation_utils``, ``seed_modes_3d``, ``plot_utils_3d`` ...) resolve from
there, so the reference's drivers import this package unchanged.
"""

import os as _os

_ref = _os.environ.get("MPF3D_REFERENCE_SRC")
if _ref and _os.path.isdir(_ref) and _ref not in __path__:
    __path__.append(_ref)
