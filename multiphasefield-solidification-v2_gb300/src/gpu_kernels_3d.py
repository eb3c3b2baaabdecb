"""
gpu_kernels_3d.py -- drop-in replacement of the reference module of the same
path (daikihatanaka0327/multiphasefield-solidification-v2, src/gpu_kernels_3d.py).

Same exported names, same call form ``kernel[blocks, threads](*args)`` (and
``kernel[blocks, threads, stream](*args)``), same argument lists and array
layout.  The kernels run as hand-written sm_103a CUDA in libmpf3d.so; the
launch geometry given by the caller is accepted and ignored because the
native kernels choose their own (z-contiguous) thread mapping.

Arrays may be any CUDA device array exposing ``__cuda_array_interface__``
(Numba device arrays, torch tensors, CuPy).  Launches are asynchronous on
the array's stream (legacy default stream when none is given), as in the
reference.  Device-side findings the reference would not detect (nf above
KMAX in the update, an unchecked APT running past mf's depth) are recorded
in a sticky word; call :func:`check_errors` to raise them.

Boundary conditions: x, y periodic; z Neumann (clamped index).
"""

import os
import sys

_PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if _PKG_ROOT not in sys.path:
    sys.path.insert(0, _PKG_ROOT)

from mpf3d import dense as _dense  # noqa: E402

# Compile-time constants of the reference (src/gpu_kernels_3d.py:20-21).
KMAX = 50
LIQ = 0

__all__ = [
    "KMAX",
    "LIQ",
    "kernel_update_nfmf_3d",
    "kernel_update_nfmf_3d_checked",
    "kernel_update_phasefield_active_3d",
    "kernel_update_phasefield_active_3d_switchable",
    "kernel_update_temp_3d",
    "check_errors",
]


class _DropInKernel:
    """Kernel object with the reference's ``kernel[blocks, threads](...)`` form."""

    def __init__(self, name, fn):
        self.__name__ = name
        self._fn = fn

    def __getitem__(self, cfg):
        if not isinstance(cfg, tuple) or len(cfg) < 2:
            raise ValueError("launch configuration must be [blocks, threads] or [blocks, threads, stream]")
        stream = cfg[2] if len(cfg) > 2 else None

        def launch(*args):
            self._fn(stream, *args)

        return launch

    def __call__(self, *args, **kwargs):
        raise ValueError("kernel launch configuration was not specified: use kernel[blocks, threads](...)")

    def __repr__(self):
        return f"<mpf3d sm_103a kernel {self.__name__}>"


def _nfmf(stream, phi, mf, nf, nx, ny, nz, number_of_grain):
    _dense.apt(phi, mf, nf, nx, ny, nz, number_of_grain, checked=False, stream=stream)


def _nfmf_checked(stream, phi, mf, nf, status, nx, ny, nz, number_of_grain):
    _dense.apt(phi, mf, nf, nx, ny, nz, number_of_grain, status=status, checked=True, stream=stream)


def _update(stream, phi, phi_new, temp, mf, nf, wij, aij, mij, n111, nx, ny, nz, number_of_grain,
            dx, dt, T_melt, Sf, eps0_sl, w0_sl, a0, delta_a, mu_a, p_round, g2_floor, ksi,
            theta_c_rad):
    _dense.update(phi, phi_new, temp, mf, nf, wij, aij, mij, n111, nx, ny, nz, number_of_grain,
                  (dx, dt, T_melt, Sf, eps0_sl, w0_sl, a0, delta_a, mu_a, p_round, g2_floor, ksi,
                   theta_c_rad), switchable=False, stream=stream)


def _update_switchable(stream, phi, phi_new, temp, mf, nf, wij, aij, mij, n111, nx, ny, nz,
                       number_of_grain, dx, dt, T_melt, Sf, eps0_sl, w0_sl, a0, delta_a, mu_a,
                       p_round, g2_floor, ksi, theta_c_rad, enable_anisotropy, enable_torque):
    _dense.update(phi, phi_new, temp, mf, nf, wij, aij, mij, n111, nx, ny, nz, number_of_grain,
                  (dx, dt, T_melt, Sf, eps0_sl, w0_sl, a0, delta_a, mu_a, p_round, g2_floor, ksi,
                   theta_c_rad), switchable=True, enable_anisotropy=int(enable_anisotropy),
                  enable_torque=int(enable_torque), stream=stream)


def _temp(stream, temp, cooling_rate, nx, ny, nz):
    _dense.temp_step(temp, cooling_rate, nx, ny, nz, stream=stream)


kernel_update_nfmf_3d = _DropInKernel("kernel_update_nfmf_3d", _nfmf)
kernel_update_nfmf_3d_checked = _DropInKernel("kernel_update_nfmf_3d_checked", _nfmf_checked)
kernel_update_phasefield_active_3d = _DropInKernel("kernel_update_phasefield_active_3d", _update)
kernel_update_phasefield_active_3d_switchable = _DropInKernel(
    "kernel_update_phasefield_active_3d_switchable", _update_switchable)
kernel_update_temp_3d = _DropInKernel("kernel_update_temp_3d", _temp)

check_errors = _dense.check_errors
