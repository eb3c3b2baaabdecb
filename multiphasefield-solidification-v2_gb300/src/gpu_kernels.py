"""
gpu_kernels.py -- drop-in replacement of the reference's 2D kernel module of
the same path (daikihatanaka0327/multiphasefield-solidification-v2,
src/gpu_kernels.py), which its 3D verification suite imports
(tests/verification_3d.py:21-25) for the two_d_limit_consistency case.

Same exported names, call form ``kernel[blocks, threads](*args)`` (and
``kernel[blocks, threads, stream](*args)``), argument lists and array layout
([N, nx, ny], y contiguous).  The kernels run as hand-written sm_103a CUDA in
libmpf3d.so; the caller's launch geometry is accepted and ignored.

Boundary conditions: x periodic; y Neumann (clamped index).  Device-side
findings (nf above KMAX, an APT deeper than mf) go to the same sticky word
as the 3D kernels; :func:`check_errors` raises them.
"""

import os
import sys

_PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if _PKG_ROOT not in sys.path:
    sys.path.insert(0, _PKG_ROOT)

from mpf3d import dense as _dense  # noqa: E402
from mpf3d import dense2d as _dense2d  # noqa: E402

from .gpu_kernels_3d import _DropInKernel  # noqa: E402

# Compile-time constants of the reference (src/gpu_kernels.py:18-19).
KMAX = 50
LIQ = 0

__all__ = ["KMAX", "LIQ", "kernel_update_nfmf", "kernel_update_phasefield_active", "kernel_update_temp",
           "check_errors"]


def _nfmf(stream, phi, mf, nf, nx, ny, number_of_grain):
    _dense2d.apt(phi, mf, nf, nx, ny, number_of_grain, stream=stream)


def _update(stream, phi, phi_new, temp, mf, nf, wij, aij, mij, n111, nx, ny, number_of_grain, dx, dt, T_melt,
            Sf, eps0_sl, w0_sl, a0, delta_a, mu_a, p_round, g2_floor, ksi, theta_c_rad):
    _dense2d.update(phi, phi_new, temp, mf, nf, wij, aij, mij, n111, nx, ny, number_of_grain,
                    (dx, dt, T_melt, Sf, eps0_sl, w0_sl, a0, delta_a, mu_a, p_round, g2_floor, ksi, theta_c_rad),
                    stream=stream)


def _temp(stream, temp, cooling_rate, nx, ny):
    _dense2d.temp_step(temp, cooling_rate, nx, ny, stream=stream)


kernel_update_nfmf = _DropInKernel("kernel_update_nfmf", _nfmf)
kernel_update_phasefield_active = _DropInKernel("kernel_update_phasefield_active", _update)
kernel_update_temp = _DropInKernel("kernel_update_temp", _temp)

check_errors = _dense.check_errors
