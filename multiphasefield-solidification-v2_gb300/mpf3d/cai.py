"""Device-array access through ``__cuda_array_interface__`` (CAI v2/v3).

Works for Numba device arrays, torch CUDA tensors and CuPy arrays alike, so
the drop-in kernels accept whatever the reference's callers hold.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

CUDA_STREAM_LEGACY = 0x1
CUDA_STREAM_PER_THREAD = 0x2


@dataclass
class DevArray:
    ptr: int
    shape: tuple
    dtype: np.dtype
    stream: int | None  # CAI stream value (None: not given)
    obj: object

    @property
    def size(self) -> int:
        n = 1
        for s in self.shape:
            n *= s
        return n


def as_dev(obj, name: str) -> DevArray:
    cai = getattr(obj, "__cuda_array_interface__", None)
    if cai is None:
        raise TypeError(f"{name}: expected a CUDA device array (an object exposing "
                        f"__cuda_array_interface__), got {type(obj).__name__}")
    shape = tuple(int(s) for s in cai["shape"])
    dtype = np.dtype(cai["typestr"])
    strides = cai.get("strides")
    if strides is not None:
        exp = []
        acc = dtype.itemsize
        for s in reversed(shape):
            exp.append(acc)
            acc *= s
        if tuple(strides) != tuple(reversed(exp)) and int(np.prod(shape)) > 1:
            raise ValueError(f"{name}: array must be C-contiguous (strides {strides})")
    ptr = int(cai["data"][0])
    return DevArray(ptr, shape, dtype, cai.get("stream"), obj)


def stream_handle(cfg_stream, arrays) -> int:
    """Stream to enqueue on: the launch-config stream if given, else the CAI
    stream of the first array that names one, else the legacy default stream."""
    if cfg_stream is not None and cfg_stream != 0:
        if hasattr(cfg_stream, "cuda_stream"):  # torch
            h = cfg_stream.cuda_stream
        elif hasattr(cfg_stream, "ptr"):  # CuPy
            h = cfg_stream.ptr
        else:  # Numba (handle is a ctypes pointer) or a raw handle
            h = getattr(cfg_stream, "handle", cfg_stream)
            h = getattr(h, "value", h)
        return int(h or 0)
    for a in arrays:
        s = a.stream
        if s is None:
            continue
        if s == CUDA_STREAM_LEGACY:
            return 0
        if s == CUDA_STREAM_PER_THREAD:
            return CUDA_STREAM_PER_THREAD
        return int(s)
    return 0
