"""``numba.cuda`` stand-in (test infrastructure): device arrays with
``__cuda_array_interface__``, ``copy_to_host`` / ``copy_to_device``,
``to_device``, ``synchronize`` and ``is_available``, on torch CUDA tensors.
Work is ordered on torch's default stream, which is the legacy default
stream the drop-in kernels launch on when an array names no other."""

from __future__ import annotations

import numpy as np
import torch


class DeviceNDArray:
    def __init__(self, tensor: torch.Tensor):
        self._t = tensor

    @property
    def __cuda_array_interface__(self):
        return self._t.__cuda_array_interface__

    @property
    def shape(self):
        return tuple(self._t.shape)

    @property
    def ndim(self):
        return self._t.dim()

    @property
    def size(self):
        return self._t.numel()

    @property
    def dtype(self):
        return np.dtype(str(self._t.dtype).replace("torch.", ""))

    def copy_to_host(self, ary=None, stream=0):
        host = self._t.cpu().numpy()
        if ary is None:
            return host
        ary[...] = host
        return ary

    def copy_to_device(self, ary, stream=0):
        src = ary._t if isinstance(ary, DeviceNDArray) else torch.from_numpy(np.ascontiguousarray(ary))
        self._t.copy_(src.reshape(self._t.shape))


def to_device(obj, stream=0, copy=True, to=None):
    arr = np.ascontiguousarray(obj)
    if to is not None:
        to.copy_to_device(arr)
        return to
    return DeviceNDArray(torch.from_numpy(arr.copy()).cuda())


def synchronize():
    torch.cuda.synchronize()


def is_available():
    return torch.cuda.is_available()
