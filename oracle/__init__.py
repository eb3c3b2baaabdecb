"""CPU oracle for the 3D multi-phase-field step (ctypes front of mpf3d_oracle.c)
and for the reference's 2D kernels (mpf2d_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py`` as the checker.  The product path
never imports it.

The C restatement follows the reference's ``src/gpu_kernels_3d.py``
(daikihatanaka0327/multiphasefield-solidification-v2) with compiled-Numba
arithmetic typing; it is pinned against golden vectors produced by running
the reference's own kernel source (``tests/golden/make_golden.py``).
"""

from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "mpf3d_oracle.c")
SRC2D = os.path.join(HERE, "mpf2d_oracle.c")
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libmpf3d_oracle.so")

KMAX = 50
SCALAR_NAMES = ["dx", "dt", "T_melt", "Sf", "eps0_sl", "w0_sl", "a0", "delta_a", "mu_a",
                "p_round", "g2_floor", "ksi", "theta_c_rad"]


class Scalars(ctypes.Structure):
    _fields_ = [("v", ctypes.c_double * 13), ("f32mask", ctypes.c_uint32)]


def build(force: bool = False) -> str:
    """Compile the oracle with gcc (OpenMP, no FP contraction)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    stale = not os.path.exists(LIB_PATH) or any(os.path.getmtime(LIB_PATH) < os.path.getmtime(f)
                                                for f in (SRC, SRC2D))
    if force or stale:
        tmp = LIB_PATH + f".tmp{os.getpid()}"
        subprocess.check_call(["gcc", "-O2", "-std=c11", "-fopenmp", "-ffp-contract=off", "-fPIC",
                               "-shared", "-o", tmp, SRC, SRC2D, "-lm"])
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        vp, i32, i64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64
        L.mpf3d_oracle_apt.argtypes = [vp, i32, i32, i32, i32, i32, vp, i32, vp, vp, i32, i32]
        L.mpf3d_oracle_apt.restype = i32
        L.mpf3d_oracle_temp.argtypes = [vp, i32, ctypes.c_double, i32, i64]
        L.mpf3d_oracle_temp.restype = None
        L.mpf3d_oracle_update.argtypes = ([vp, vp, i32, vp, i32, vp, i32, vp, vp, vp, vp, vp]
                                          + [i32] * 4 + [ctypes.POINTER(Scalars)] + [i32] * 4)
        L.mpf3d_oracle_update.restype = i32
        L.mpf2d_oracle_apt.argtypes = [vp, i32, i32, i32, i32, vp, i32, vp]
        L.mpf2d_oracle_apt.restype = i32
        L.mpf2d_oracle_update.argtypes = ([vp, vp, i32, vp, i32, vp, vp, vp, vp, vp, vp] + [i32] * 3
                                          + [ctypes.POINTER(Scalars), i32])
        L.mpf2d_oracle_update.restype = i32
        _LIB = L
    return _LIB


def _ptr(a: np.ndarray):
    assert a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.c_void_p)


def make_scalars(values, f32) -> Scalars:
    """values: dict or sequence in SCALAR_NAMES order; f32: bool or per-name mask."""
    if isinstance(values, dict):
        values = [values[k] for k in SCALAR_NAMES]
    s = Scalars()
    mask = 0
    for i, v in enumerate(values):
        is32 = f32[i] if isinstance(f32, (list, tuple, np.ndarray)) else bool(f32)
        s.v[i] = float(np.float32(v)) if is32 else float(v)
        mask |= (1 << i) if is32 else 0
    s.f32mask = mask
    return s


def apt(phi: np.ndarray, mf: np.ndarray, nf: np.ndarray, status=None, checked=True, kmax=KMAX) -> int:
    N, nx, ny, nz = phi.shape
    st = status if status is not None else np.zeros(2, np.int32)
    return lib().mpf3d_oracle_apt(_ptr(phi), int(phi.dtype == np.float64), N, nx, ny, nz, _ptr(mf),
                                  mf.shape[0], _ptr(nf), _ptr(st), int(checked), kmax)


def temp_step(temp: np.ndarray, rate: float, rate_f32: bool) -> None:
    lib().mpf3d_oracle_temp(_ptr(temp), int(temp.dtype == np.float64), float(rate), int(rate_f32),
                            temp.size)


def update(phi, phi_new, temp, mf, nf, wij, aij, mij, n111, scalars: Scalars, switchable=False,
           aniso=1, torque=1, kmax=KMAX) -> int:
    N, nx, ny, nz = phi.shape
    assert phi_new.dtype == phi.dtype
    for a in (wij, aij, mij, n111):
        assert a.dtype == np.float32
    return lib().mpf3d_oracle_update(
        _ptr(phi), _ptr(phi_new), int(phi.dtype == np.float64), _ptr(temp),
        int(temp.dtype == np.float64), _ptr(mf), mf.shape[0], _ptr(nf), _ptr(wij), _ptr(aij),
        _ptr(mij), _ptr(n111), N, nx, ny, nz, ctypes.byref(scalars), int(switchable), int(aniso),
        int(torque), kmax)


def run(phi0, temp0, wij, aij, mij, n111, scalars: Scalars, steps, *, cooling_rate=0.0,
        rate_f32=True, cooling=True, checked=True, switchable=True, aniso=1, torque=1,
        kmax=KMAX, record=False):
    """Run `steps` reference steps (temperature, APT, update, swap) on the CPU."""
    phi = np.ascontiguousarray(phi0).copy()
    phi_new = phi.copy()
    temp = np.ascontiguousarray(temp0).copy()
    N, nx, ny, nz = phi.shape
    mf = np.zeros((max(N, kmax), nx, ny, nz), np.int32)
    nf = np.zeros((nx, ny, nz), np.int32)
    hist = []
    for _ in range(steps):
        if cooling:
            temp_step(temp, cooling_rate, rate_f32)
        st = np.zeros(2, np.int32)
        rc = apt(phi, mf, nf, st, checked=checked, kmax=kmax)
        if rc != 0 or st[0] != 0:
            raise RuntimeError(f"oracle APT failed rc={rc} status={st.tolist()}")
        rc = update(phi, phi_new, temp, mf, nf, wij, aij, mij, n111, scalars, switchable, aniso,
                    torque, kmax)
        if rc != 0:
            raise RuntimeError(f"oracle update failed rc={rc}")
        phi, phi_new = phi_new, phi
        if record:
            hist.append((phi.copy(), nf.copy(), mf.copy(), st.copy(), temp.copy()))
    return (phi, temp, nf, mf, hist) if record else (phi, temp, nf, mf)


# --- 2D kernels (src/gpu_kernels.py) -------------------------------------

def apt2d(phi: np.ndarray, mf: np.ndarray, nf: np.ndarray) -> int:
    """kernel_update_nfmf (src/gpu_kernels.py:337-358); -1 if mf is too shallow."""
    N, nx, ny = phi.shape
    return lib().mpf2d_oracle_apt(_ptr(phi), int(phi.dtype == np.float64), N, nx, ny, _ptr(mf), mf.shape[0],
                                  _ptr(nf))


def update2d(phi, phi_new, temp, mf, nf, wij, aij, mij, n111, scalars: Scalars, kmax=KMAX) -> int:
    """kernel_update_phasefield_active (src/gpu_kernels.py:361-517)."""
    N, nx, ny = phi.shape
    assert phi_new.dtype == phi.dtype
    for a in (wij, aij, mij, n111):
        assert a.dtype == np.float32
    return lib().mpf2d_oracle_update(
        _ptr(phi), _ptr(phi_new), int(phi.dtype == np.float64), _ptr(temp), int(temp.dtype == np.float64),
        _ptr(mf), _ptr(nf), _ptr(wij), _ptr(aij), _ptr(mij), _ptr(n111), N, nx, ny, ctypes.byref(scalars), kmax)


def run2d(phi0, temp0, wij, aij, mij, n111, scalars: Scalars, steps, *, cooling_rate=0.0, rate_f32=True,
          cooling=True, depth=None, kmax=KMAX):
    """Run `steps` 2D reference steps (temperature, APT, update, swap), in the
    order of the reference's run_2d_simulation (tests/verification_3d.py:939-1000)."""
    phi = np.ascontiguousarray(phi0).copy()
    phi_new = phi.copy()
    temp = np.ascontiguousarray(temp0).copy()
    N, nx, ny = phi.shape
    mf = np.zeros((depth or max(N, 18), nx, ny), np.int32)
    nf = np.zeros((nx, ny), np.int32)
    for _ in range(steps):
        if cooling and cooling_rate != 0.0:
            temp_step(temp, cooling_rate, rate_f32)
        if apt2d(phi, mf, nf) != 0:
            raise RuntimeError("oracle 2D APT: mf too shallow")
        rc = update2d(phi, phi_new, temp, mf, nf, wij, aij, mij, n111, scalars, kmax)
        if rc != 0:
            raise RuntimeError(f"oracle 2D update failed rc={rc}")
        phi, phi_new = phi_new, phi
    return phi, temp, nf, mf
