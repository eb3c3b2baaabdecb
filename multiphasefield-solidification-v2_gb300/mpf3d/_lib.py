"""ctypes binding of libmpf3d.so (the C ABI declared in include/mpf3d.h).

There is no fallback: if the library is missing or fails to load, every
entry point raises.
"""

from __future__ import annotations

import ctypes
import os

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libmpf3d.so")

MPF3D_OK = 0
STEP_MULTI_LIST = 1  # MPF3D_STEP_MULTI_LIST
STEP_SWEEP_TMA = 2  # MPF3D_STEP_SWEEP_TMA
ERRORS = {-1: "bad argument", -2: "bad dtype", -3: "CUDA launch/call failed", -4: "size above limit"}

DEV_BITS = {1: "unchecked APT needed more rows than mf has (MPF3D_DEV_MF_DEPTH)",
            2: "update met nf > KMAX (MPF3D_DEV_NF_GT_KMAX)",
            4: "update met an mf id outside [0, N) (MPF3D_DEV_BAD_ID)",
            8: "compact stepper: more phases than slots (MPF3D_DEV_SLOT_OVERFLOW)",
            16: "compact conversion met a negative or NaN phi (MPF3D_DEV_BAD_INPUT)",
            32: "tcgen05 GEMM: a bounded wait ran out, outputs written as NaN (MPF3D_DEV_GEMM_ABORT)",
            64: "compact step: a TMA staging copy did not land in time (MPF3D_DEV_STAGING_TIMEOUT)"}

_VP = ctypes.c_void_p
_I32 = ctypes.c_int
_I64 = ctypes.c_int64
_F64 = ctypes.c_double


class Scalars(ctypes.Structure):
    """mpf3d_scalars: the 13 float arguments + float32 mask."""
    _fields_ = [("v", ctypes.c_double * 13), ("f32mask", ctypes.c_uint32)]


class Tuning(ctypes.Structure):
    """mpf3d_tuning: launch shape of the compact step."""
    _fields_ = [("sweep_zb", ctypes.c_int32), ("sweep_by", ctypes.c_int32),
                ("general_blocks_per_sm", ctypes.c_int32), ("general_threads", ctypes.c_int32),
                ("iface_blocks_per_sm", ctypes.c_int32), ("iface_threads", ctypes.c_int32)]


class Metrics(ctypes.Structure):
    """mpf3d_metrics: reductions of compute_metrics_3d over a compact state."""
    _fields_ = [("solid_sum", ctypes.c_double), ("sum_err_max", ctypes.c_double), ("phi_min", ctypes.c_double),
                ("phi_max", ctypes.c_double), ("front_sum", ctypes.c_double), ("front_sq_sum", ctypes.c_double),
                ("front_max", ctypes.c_double), ("nan_count", ctypes.c_int64), ("front_columns", ctypes.c_int64),
                ("nf_max", ctypes.c_int32), ("reserved", ctypes.c_int32)]


_F32 = ctypes.c_float
_U32 = ctypes.c_uint32

# name -> (restype, argtypes)
_SIGS = {
    "mpf3d_host_device_pointer": (_I32, [_VP, ctypes.POINTER(ctypes.c_void_p)]),
    "mpf3d_version": (_I32, []),
    "mpf3d_dense_apt": (_I32, [_VP, _I32, _I32, _I32, _I32, _I32, _VP, _I32, _VP, _VP, _I32, _VP, _VP]),
    "mpf3d_dense_update": (_I32, [_VP, _VP, _I32, _VP, _I32, _VP, _I32, _VP, _VP, _VP, _VP, _VP,
                                  _I32, _I32, _I32, _I32, ctypes.POINTER(Scalars), _I32, _I32, _I32,
                                  _VP, _VP]),
    "mpf3d_dense_temp": (_I32, [_VP, _I32, _F64, _I32, _I64, _VP]),
    "mpf2d_dense_apt": (_I32, [_VP, _I32, _I32, _I32, _I32, _VP, _I32, _VP, _VP, _VP]),
    "mpf2d_dense_update": (_I32, [_VP, _VP, _I32, _VP, _I32, _VP, _I32, _VP, _VP, _VP, _VP, _VP,
                                  _I32, _I32, _I32, ctypes.POINTER(Scalars), _VP, _VP]),
    "mpf2d_dense_temp": (_I32, [_VP, _I32, _F64, _I32, _I32, _I32, _VP]),
    "mpf3d_compact_metrics": (_I32, [_VP, _VP, _VP, _I32, _I32, _I32, _I32, _I32, _F32, _VP, _VP, _VP, _VP]),
    "mpf3d_compact_slice": (_I32, [_VP, _VP, _VP, _I32, _I32, _I32, _I32, _I32, _I32, _VP, _VP, _VP, _VP]),
    "mpf3d_compact_pack_scratch_len": (_I64, [_I64]),
    "mpf3d_compact_pack": (_I32, [_VP, _VP, _VP, _I32, _I64, _VP, _VP, _VP, _VP, _I64, _VP, _VP]),
    "mpf3d_compact_unpack": (_I32, [_VP, _VP, _VP, _I64, _I32, _I64, _VP, _VP, _VP, _VP, _VP]),
    "mpf3d_batched_init_sphere": (_I32, [_VP, _I32, _U32, _F64, _F64, _VP, _VP, _I32, _I32, _VP, _VP, _VP, _VP]),
    "mpf3d_batched_ray_radii": (_I32, [_VP, _VP, _VP, _I32, _VP, _I32, _U32, _I32, _VP, _VP, _I32, _F64, _F64,
                                       _VP, _VP]),
    "mpf3d_compact_from_dense": (_I32, [_VP, _I32, _I32, _I32, _I32, _I32, _I32, _VP, _VP, _VP, _VP, _VP]),
    "mpf3d_compact_to_dense": (_I32, [_VP, _VP, _VP, _I32, _I32, _I32, _I32, _I32, _VP, _I32, _VP]),
    "mpf3d_compact_active_count": (_I32, [_VP, _VP, _I32, _I32, _I32, _I32, _VP, _VP]),
    "mpf3d_streams_prepare": (_I32, [_VP]),
    "mpf3d_compact_step": (_I32, [_VP, _VP, _VP, _VP, _VP, _VP, _I32, _I32, _VP, _F64, _VP, _VP, _VP, _VP,
                                  _I32, _I32, _I32, _I32, ctypes.POINTER(Scalars), _I32, _I32, _I32,
                                  _VP, _VP, _I32, _VP, _VP]),
    "mpf3d_compact_to_dense_view": (_I32, [_VP, _VP, _VP, _I32, ctypes.c_uint32, ctypes.c_uint32, _I32, _I32,
                                           _I32, _I32, _VP, _I32, _VP]),
    "mpf3d_batched_init_bicrystal": (_I32, [_VP, _I32, ctypes.c_uint32, _F64, _F64, _VP, _VP, _VP, _VP, _VP]),
    "mpf3d_batched_step": (_I32, [_VP, _VP, _VP, _VP, _VP, _VP, _I32, _I32, _VP, _I32, _I32, ctypes.c_uint32,
                                  _VP, _VP, _VP, _VP, _I32, ctypes.POINTER(Scalars), _I32, _I32, _I32, _VP,
                                  _VP, _I32, _VP, _VP, _I32]),
    "mpf3d_batched_step_tuned": (_I32, [_VP, _VP, _VP, _VP, _VP, _VP, _I32, _I32, _VP, _I32, _I32, ctypes.c_uint32,
                                        _VP, _VP, _VP, _VP, _I32, ctypes.POINTER(Scalars), _I32, _I32, _I32, _VP,
                                        _VP, _I32, _VP, _VP, _I32, _VP, _VP]),
    "mpf3d_batched_tile_flags_len": (_I64, [_I32]),
    "mpf3d_batched_fronts": (_I32, [_VP, _VP, _VP, _I32, _VP, _I32, ctypes.c_uint32, _VP, _VP]),
    "mpf3d_batched_gb_rows": (_I32, [_VP, _VP, _VP, _I32, _VP, _I32, ctypes.c_uint32, _VP, _VP, _VP]),
    "mpf3d_compact_init_owner": (_I32, [_VP, _I32, _VP, _I32, _I32, _I32, _I32, _VP, _VP, _VP, _VP]),
    "mpf3d_gemm_bf16": (_I32, [_I32, _I32, _I32, _VP, _I64, _I64, _VP, _I64, _I64, _VP, _I32, _VP, _VP, _I32,
                               _I32, _I32, _VP, _VP]),
    "mpf3d_gemm_bf16_mma": (_I32, [_I32, _I32, _I32, _VP, _I64, _I64, _VP, _I64, _I64, _VP, _I32, _VP, _VP, _I32,
                               _I32, _I32, _VP]),
    "mpf3d_gemm_bf16_tc5": (_I32, [_I32, _I32, _I32, _VP, _I64, _VP, _I64, _VP, _I32, _VP, _VP, _I32, _I32, _I32,
                                   _VP, _VP]),
    "mpf3d_gemm_bf16_tc5_strided": (_I32, [_I32, _I32, _I32, _VP, _I64, _I64, _VP, _I64, _I64, _VP, _I32, _VP, _VP,
                                           _I32, _I32, _I32, _VP, _VP]),
    "mpf3d_gemm_bf16_tc5_held": (_I32, [_I32, _I32, _I32, _VP, _I64, _VP, _I64, _VP, _I32, _VP, ctypes.c_uint64,
                                        _VP]),
    "mpf3d_act_backward": (_I32, [_VP, _VP, _I32, _I64, _VP, _VP, _VP]),
    "mpf3d_colsum": (_I32, [_VP, _I32, _I32, _I32, _VP, _VP]),
    "mpf3d_mse": (_I32, [_VP, _I32, _VP, _I32, _I32, _VP, _VP, _VP, _VP]),
    "mpf3d_adam": (_I32, [_VP, _VP, _VP, _VP, _VP, _I64, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                          ctypes.c_float, _I32, ctypes.c_float, _VP]),
    "mpf3d_f32_to_bf16": (_I32, [_VP, _VP, _I64, _VP]),
    "mpf3d_compact_step_tuned": (_I32, [_VP, _VP, _VP, _VP, _VP, _VP, _I32, _I32, _VP, _F64, _VP, _VP, _VP, _VP,
                                        _I32, _I32, _I32, _I32, ctypes.POINTER(Scalars), _I32, _I32, _I32,
                                        _VP, _VP, _I32, _VP, _VP, ctypes.POINTER(Tuning), _VP, _I32]),
    "mpf3d_compact_step_clocked": (_I32, [_VP, _VP, _VP, _VP, _VP, _VP, _I32, _I32, _VP, _VP, _F64, _F64, _VP, _VP,
                                          _VP, _VP, _I32, _I32, _I32, _I32, ctypes.POINTER(Scalars), _I32, _I32,
                                          _I32, _VP, _VP, _I32, _VP, _VP, ctypes.POINTER(Tuning), _VP, _I32]),
    "mpf3d_compact_tile_flags_len": (_I64, [_I32, _I32, _I32]),
    "mpf3d_compact_step_noalloc": (_I32, [_VP, _VP, _VP, _VP, _VP, _VP, _I32, _I32, _VP, _F64, _VP, _VP,
                                          _VP, _VP, _I32, _I32, _I32, _I32, ctypes.POINTER(Scalars),
                                          _I32, _I32, _I32, _VP, _VP]),
}

_LIB = None


class LibraryMissing(RuntimeError):
    pass


def library_path() -> str:
    """The library to load: $MPF3D_LIBRARY when set (another build of the
    same C ABI), else the in-tree build next to this module."""
    return os.environ.get("MPF3D_LIBRARY") or LIB_PATH


def lib():
    global _LIB
    if _LIB is None:
        path = library_path()
        if not os.path.exists(path):
            raise LibraryMissing(f"{path} is not built: run `python -c \"import __graft_entry__ as g; "
                                 "g.build()\"` (or multiphasefield-solidification-v2_gb300/build.py)")
        L = ctypes.CDLL(path)
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


def exported_symbols():
    """Names the binding expects the library to export."""
    return list(_SIGS)


def check(rc: int, what: str) -> None:
    if rc != MPF3D_OK:
        raise RuntimeError(f"{what} failed: {ERRORS.get(rc, rc)}")


def describe_dev_error(word: int) -> str:
    return "; ".join(msg for bit, msg in DEV_BITS.items() if word & bit) or "none"


def host_device_pointer(t) -> int:
    """Device address of a pinned (page-locked) CPU tensor's memory, so that a
    kernel can read or write it over the CPU-GPU link without a staging copy."""
    d = ctypes.c_void_p()
    check(lib().mpf3d_host_device_pointer(t.data_ptr(), ctypes.byref(d)), "host_device_pointer")
    return int(d.value)
