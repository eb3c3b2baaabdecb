"""Host side of the 2D kernels: argument checks, scalar typing and launches of
the C ABI (``mpf2d_dense_*``) on the caller's stream.

These functions back the kernel objects of ``src/gpu_kernels.py``; their
argument lists are the reference's 2D kernels' (src/gpu_kernels.py:337-525).
"""

from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .cai import as_dev, stream_handle
from .dense import _DT, _err_word, _i32, _is_f32, make_scalars


def _dims(phi, nx, ny, number_of_grain):
    if len(phi.shape) != 3:
        raise ValueError(f"phi must be 3-D [N, nx, ny], got shape {phi.shape}")
    N, sx, sy = phi.shape
    if (int(nx), int(ny)) != (sx, sy):
        raise ValueError(f"nx, ny = {(nx, ny)} do not match phi's shape {phi.shape}")
    if int(number_of_grain) != N:
        raise ValueError(f"number_of_grain={number_of_grain} does not match phi.shape[0]={N}")
    if phi.dtype not in _DT:
        raise TypeError(f"phi must be float32 or float64, got {phi.dtype}")
    return N, sx, sy


def _mf(M, nx, ny):
    _i32(M, "mf")
    if len(M.shape) != 3 or M.shape[1:] != (nx, ny):
        raise ValueError(f"mf must have shape [depth, {nx}, {ny}], got {M.shape}")


def apt(phi, mf, nf, nx, ny, number_of_grain, stream=None):
    P, M, F = as_dev(phi, "phi"), as_dev(mf, "mf"), as_dev(nf, "nf")
    N, nx, ny = _dims(P, nx, ny, number_of_grain)
    _mf(M, nx, ny)
    _i32(F, "nf", (nx, ny))
    h = stream_handle(stream, [P, M, F])
    rc = _lib.lib().mpf2d_dense_apt(P.ptr, _DT[P.dtype], N, nx, ny, M.ptr, M.shape[0], F.ptr,
                                    _err_word().data_ptr(), h or None)
    _lib.check(rc, "2D APT")


def update(phi, phi_new, temp, mf, nf, wij, aij, mij, n111, nx, ny, number_of_grain, scalars, stream=None):
    P, Q, T = as_dev(phi, "phi"), as_dev(phi_new, "phi_new"), as_dev(temp, "temp")
    M, F = as_dev(mf, "mf"), as_dev(nf, "nf")
    W, A, Mi, U = (as_dev(x, n) for x, n in ((wij, "wij"), (aij, "aij"), (mij, "mij"), (n111, "n111")))
    N, nx, ny = _dims(P, nx, ny, number_of_grain)
    if N < 2:
        raise ValueError("the 2D update needs at least one solid grain (number_of_grain >= 2)")
    if Q.shape != P.shape or Q.dtype != P.dtype:
        raise ValueError(f"phi_new must match phi ({P.shape}, {P.dtype}); got ({Q.shape}, {Q.dtype})")
    if Q.ptr == P.ptr:
        raise ValueError("phi_new must not alias phi")
    if T.shape != (nx, ny) or T.dtype not in _DT:
        raise ValueError(f"temp must be float32/float64 [{nx}, {ny}], got {T.shape} {T.dtype}")
    _mf(M, nx, ny)
    _i32(F, "nf", (nx, ny))
    for X, nm in ((W, "wij"), (A, "aij"), (Mi, "mij")):
        if X.dtype != np.float32 or X.shape != (N, N):
            raise TypeError(f"{nm} must be float32 [{N}, {N}], got {X.dtype} {X.shape}")
    if U.dtype != np.float32 or U.shape != (N, 8, 3):
        raise TypeError(f"n111 must be float32 [{N}, 8, 3], got {U.dtype} {U.shape}")
    sc = scalars if isinstance(scalars, _lib.Scalars) else make_scalars(scalars)
    h = stream_handle(stream, [P, Q, T, M, F])
    rc = _lib.lib().mpf2d_dense_update(P.ptr, Q.ptr, _DT[P.dtype], T.ptr, _DT[T.dtype], M.ptr, M.shape[0], F.ptr,
                                       W.ptr, A.ptr, Mi.ptr, U.ptr, N, nx, ny, ctypes.byref(sc),
                                       _err_word().data_ptr(), h or None)
    _lib.check(rc, "2D phase update")


def temp_step(temp, cooling_rate, nx, ny, stream=None):
    T = as_dev(temp, "temp")
    if T.shape != (int(nx), int(ny)) or T.dtype not in _DT:
        raise ValueError(f"temp must be float32/float64 [{nx}, {ny}], got {T.shape} {T.dtype}")
    h = stream_handle(stream, [T])
    rc = _lib.lib().mpf2d_dense_temp(T.ptr, _DT[T.dtype], float(cooling_rate), int(_is_f32(cooling_rate)),
                                     int(nx), int(ny), h or None)
    _lib.check(rc, "2D temperature update")
