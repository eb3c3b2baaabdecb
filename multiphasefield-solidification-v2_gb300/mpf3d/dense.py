"""Host side of the dense drop-in tier: argument checks, scalar typing and
launches of the C ABI (``mpf3d_dense_*``) on the caller's stream.

These functions back the kernel objects of ``src/gpu_kernels_3d.py``; their
argument lists are the reference kernels' (src/gpu_kernels_3d.py:462-838).
"""

from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .cai import as_dev, stream_handle

KMAX = 50
LIQ = 0
SCALAR_NAMES = ("dx", "dt", "T_melt", "Sf", "eps0_sl", "w0_sl", "a0", "delta_a", "mu_a",
                "p_round", "g2_floor", "ksi", "theta_c_rad")

_DT = {np.dtype(np.float32): 0, np.dtype(np.float64): 1}
_ERR = {}


def _err_word():
    """Per-device int32 word that the kernels OR their device-side findings into."""
    import torch

    dev = torch.cuda.current_device()
    w = _ERR.get(dev)
    if w is None:
        w = torch.zeros(1, dtype=torch.int32, device=f"cuda:{dev}")
        _ERR[dev] = w
    return w


def device_error(clear: bool = True) -> int:
    """Synchronise and return (optionally clearing) the sticky device error bits."""
    import torch

    w = _err_word()
    torch.cuda.synchronize()
    v = int(w.item())
    if clear:
        w.zero_()
    return v


def check_errors() -> None:
    v = device_error(clear=True)
    if v:
        raise RuntimeError("mpf3d device error: " + _lib.describe_dev_error(v))


def _is_f32(x) -> bool:
    return isinstance(x, np.float32)


def make_scalars(values) -> _lib.Scalars:
    """13 kernel scalars -> mpf3d_scalars, recording which were float32."""
    if len(values) != 13:
        raise TypeError(f"expected 13 floating-point kernel arguments, got {len(values)}")
    s = _lib.Scalars()
    mask = 0
    for i, v in enumerate(values):
        if isinstance(v, (np.ndarray,)) and v.shape == ():
            v = v[()]
        if _is_f32(v):
            mask |= 1 << i
            s.v[i] = float(v)
        elif isinstance(v, (float, int, np.floating, np.integer)) and not isinstance(v, bool):
            s.v[i] = float(v)
        else:
            raise TypeError(f"argument {SCALAR_NAMES[i]} must be a float, got {type(v).__name__}")
    s.f32mask = mask
    return s


def _dims(phi, nx, ny, nz, number_of_grain):
    if len(phi.shape) != 4:
        raise ValueError(f"phi must be 4-D [N, nx, ny, nz], got shape {phi.shape}")
    N, sx, sy, sz = phi.shape
    if (int(nx), int(ny), int(nz)) != (sx, sy, sz):
        raise ValueError(f"nx, ny, nz = {(nx, ny, nz)} do not match phi's shape {phi.shape}")
    if int(number_of_grain) != N:
        raise ValueError(f"number_of_grain={number_of_grain} does not match phi.shape[0]={N}")
    if phi.dtype not in _DT:
        raise TypeError(f"phi must be float32 or float64, got {phi.dtype}")
    return N, sx, sy, sz


def _i32(a: "DevArray", name: str, shape=None):
    if a.dtype != np.int32:
        raise TypeError(f"{name} must be int32, got {a.dtype}")
    if shape is not None and a.shape != shape:
        raise ValueError(f"{name} must have shape {shape}, got {a.shape}")


def apt(phi, mf, nf, nx, ny, nz, number_of_grain, status=None, checked=False, stream=None):
    P, M, F = as_dev(phi, "phi"), as_dev(mf, "mf"), as_dev(nf, "nf")
    N, nx, ny, nz = _dims(P, nx, ny, nz, number_of_grain)
    _i32(M, "mf")
    if len(M.shape) != 4 or M.shape[1:] != (nx, ny, nz):
        raise ValueError(f"mf must have shape [depth, {nx}, {ny}, {nz}], got {M.shape}")
    _i32(F, "nf", (nx, ny, nz))
    arrs = [P, M, F]
    st = 0
    if checked:
        S = as_dev(status, "status")
        _i32(S, "status")
        if S.size < 2:
            raise ValueError("status must hold at least 2 int32 entries")
        st = S.ptr
        arrs.append(S)
    h = stream_handle(stream, arrs)
    rc = _lib.lib().mpf3d_dense_apt(P.ptr, _DT[P.dtype], N, nx, ny, nz, M.ptr, M.shape[0], F.ptr,
                                    st or None, int(bool(checked)), _err_word().data_ptr(), h or None)
    _lib.check(rc, "APT")


def update(phi, phi_new, temp, mf, nf, wij, aij, mij, n111, nx, ny, nz, number_of_grain, scalars,
           switchable=False, enable_anisotropy=1, enable_torque=1, stream=None):
    P, Q, T = as_dev(phi, "phi"), as_dev(phi_new, "phi_new"), as_dev(temp, "temp")
    M, F = as_dev(mf, "mf"), as_dev(nf, "nf")
    W, A, Mi, U = (as_dev(x, n) for x, n in ((wij, "wij"), (aij, "aij"), (mij, "mij"), (n111, "n111")))
    N, nx, ny, nz = _dims(P, nx, ny, nz, number_of_grain)
    if Q.shape != P.shape or Q.dtype != P.dtype:
        raise ValueError(f"phi_new must match phi ({P.shape}, {P.dtype}); got ({Q.shape}, {Q.dtype})")
    if Q.ptr == P.ptr:
        raise ValueError("phi_new must not alias phi")
    if T.shape != (nx, ny, nz) or T.dtype not in _DT:
        raise ValueError(f"temp must be float32/float64 [{nx}, {ny}, {nz}], got {T.shape} {T.dtype}")
    _i32(M, "mf")
    if len(M.shape) != 4 or M.shape[1:] != (nx, ny, nz):
        raise ValueError(f"mf must have shape [depth, {nx}, {ny}, {nz}], got {M.shape}")
    _i32(F, "nf", (nx, ny, nz))
    for X, nm in ((W, "wij"), (A, "aij"), (Mi, "mij")):
        if X.dtype != np.float32 or X.shape != (N, N):
            raise TypeError(f"{nm} must be float32 [{N}, {N}] (as build_interaction_matrices "
                            f"returns it), got {X.dtype} {X.shape}")
    if U.dtype != np.float32 or U.shape != (N, 8, 3):
        raise TypeError(f"n111 must be float32 [{N}, 8, 3], got {U.dtype} {U.shape}")
    sc = scalars if isinstance(scalars, _lib.Scalars) else make_scalars(scalars)
    h = stream_handle(stream, [P, Q, T, M, F])
    rc = _lib.lib().mpf3d_dense_update(
        P.ptr, Q.ptr, _DT[P.dtype], T.ptr, _DT[T.dtype], M.ptr, M.shape[0], F.ptr, W.ptr, A.ptr,
        Mi.ptr, U.ptr, N, nx, ny, nz, ctypes.byref(sc), int(bool(switchable)),
        int(enable_anisotropy), int(enable_torque), _err_word().data_ptr(), h or None)
    _lib.check(rc, "phase update")


def temp_step(temp, cooling_rate, nx, ny, nz, stream=None):
    T = as_dev(temp, "temp")
    if T.shape != (int(nx), int(ny), int(nz)) or T.dtype not in _DT:
        raise ValueError(f"temp must be float32/float64 [{nx}, {ny}, {nz}], got {T.shape} {T.dtype}")
    h = stream_handle(stream, [T])
    rc = _lib.lib().mpf3d_dense_temp(T.ptr, _DT[T.dtype], float(cooling_rate),
                                     int(_is_f32(cooling_rate)), T.size, h or None)
    _lib.check(rc, "temperature update")
