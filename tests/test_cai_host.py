"""Host logic of the drop-in tier's device-array access (no GPU): the
``__cuda_array_interface__`` reader and the choice of the launch stream for
Numba-, torch- and CuPy-style stream objects."""
import ctypes

import numpy as np
import pytest


class FakeDeviceArray:
    def __init__(self, shape, typestr="<f4", strides=None, stream=None, ptr=0x1000):
        self.__cuda_array_interface__ = {"shape": shape, "typestr": typestr, "data": (ptr, False),
                                         "strides": strides, "version": 3}
        if stream is not None:
            self.__cuda_array_interface__["stream"] = stream


def test_contiguous_arrays_are_accepted_and_described():
    from mpf3d.cai import as_dev
    a = as_dev(FakeDeviceArray((3, 4, 5)), "phi")
    assert (a.ptr, a.shape, a.dtype, a.size) == (0x1000, (3, 4, 5), np.dtype(np.float32), 60)
    b = as_dev(FakeDeviceArray((3, 4), "<f8", strides=(32, 8)), "phi")
    assert b.dtype == np.float64


def test_strided_or_foreign_objects_are_refused():
    from mpf3d.cai import as_dev
    with pytest.raises(ValueError):
        as_dev(FakeDeviceArray((3, 4), strides=(4, 12)), "phi")
    with pytest.raises(TypeError):
        as_dev(np.zeros(3), "phi")


class TorchLikeStream:
    cuda_stream = 0xABC


class CupyLikeStream:
    ptr = 0xDEF


class NumbaLikeStream:
    handle = ctypes.c_void_p(0x123)


@pytest.mark.parametrize("stream,want", [(TorchLikeStream(), 0xABC), (CupyLikeStream(), 0xDEF),
                                         (NumbaLikeStream(), 0x123), (0x77, 0x77)])
def test_launch_stream_objects(stream, want):
    from mpf3d.cai import stream_handle
    assert stream_handle(stream, []) == want


def test_stream_from_the_arrays_interface():
    from mpf3d.cai import CUDA_STREAM_LEGACY, CUDA_STREAM_PER_THREAD, as_dev, stream_handle
    a = as_dev(FakeDeviceArray((2,), stream=0x55), "a")
    none = as_dev(FakeDeviceArray((2,)), "b")
    assert stream_handle(None, [none, a]) == 0x55
    assert stream_handle(None, [as_dev(FakeDeviceArray((2,), stream=CUDA_STREAM_LEGACY), "c")]) == 0
    assert stream_handle(None, [as_dev(FakeDeviceArray((2,), stream=CUDA_STREAM_PER_THREAD), "d")]) == 2
    assert stream_handle(None, [none]) == 0
    assert stream_handle(0, [a]) == 0x55
