"""Typing-faithful CPU stand-in for the parts of ``numba.cuda`` that the
reference's 3D and 2D kernels use, so that the reference's own kernel source can be
executed on the host to produce golden vectors.

Test infrastructure only: nothing in the product imports this module.

Why a shim instead of ``NUMBA_ENABLE_CUDASIM``
----------------------------------------------
Numba is not installed here.  Its CUDA simulator would also round differently
from a compiled kernel: under NumPy 2 (NEP 50) ``np.float32 * 2.0`` stays
float32, while compiled Numba types every Python float literal as float64 and
promotes ``float32 op float64`` to float64.  This shim reproduces the compiled
typing rules that the reference kernels depend on:

* float32 values (elements of float32 arrays, float32 scalar arguments,
  ``float32(...)`` casts and ``cuda.local.array(..., float32)`` elements) are
  :class:`F32` objects.  ``F32 op F32`` is a float32 operation (computed in
  double and rounded once, which is the correctly rounded float32 result for
  + - * / and sqrt); ``F32 op float`` is a float64 operation.
* ``math.sqrt/tan/acos/tanh`` of an F32 return F32 (Numba calls the float32
  libm variant); of a float they return float.
* ``max(a, b)`` of mixed float32/float64 arguments returns float64, as Numba
  unifies the argument types.
* elements of ``wij`` read as float64: in both reference update kernels the
  variables that receive them (``wik``/``wjk``) are also assigned ``w_sl``,
  whose type unifies to float64, so Numba holds them in float64.
* Python floats are IEEE binary64 with no fused multiply-add, which is what
  Numba's NVVM pipeline emits without ``fastmath``.

The one operation that is not bit-faithful is the float32 ``tan`` of a float32
argument (libdevice ``tanf`` versus a correctly rounded value); it only enters
through ``tan(a0)`` when ``a0`` is passed as float32.
"""

from __future__ import annotations

import importlib.util
import itertools
import math as _math
import sys
import types

import numpy as np


def _r32(x: float) -> float:
    return float(np.float32(x))


class F32:
    """A float32 scalar with compiled-Numba promotion rules."""

    __slots__ = ("v",)

    def __init__(self, v):
        self.v = v

    # --- arithmetic -----------------------------------------------------
    def _bin(self, o, op, rev=False):
        if isinstance(o, F32):
            a, b = (o.v, self.v) if rev else (self.v, o.v)
            return F32(_r32(op(a, b)))
        o = float(o)
        a, b = (o, self.v) if rev else (self.v, o)
        return op(a, b)

    def __add__(self, o):
        return self._bin(o, lambda a, b: a + b)

    def __radd__(self, o):
        return self._bin(o, lambda a, b: a + b, True)

    def __sub__(self, o):
        return self._bin(o, lambda a, b: a - b)

    def __rsub__(self, o):
        return self._bin(o, lambda a, b: a - b, True)

    def __mul__(self, o):
        return self._bin(o, lambda a, b: a * b)

    def __rmul__(self, o):
        return self._bin(o, lambda a, b: a * b, True)

    def __truediv__(self, o):
        return self._bin(o, _div)

    def __rtruediv__(self, o):
        return self._bin(o, _div, True)

    def __neg__(self):
        return F32(-self.v)

    def __abs__(self):
        return F32(abs(self.v))

    # --- comparisons ----------------------------------------------------
    def _val(self, o):
        return o.v if isinstance(o, F32) else float(o)

    def __lt__(self, o):
        return self.v < self._val(o)

    def __le__(self, o):
        return self.v <= self._val(o)

    def __gt__(self, o):
        return self.v > self._val(o)

    def __ge__(self, o):
        return self.v >= self._val(o)

    def __eq__(self, o):
        return self.v == self._val(o)

    def __ne__(self, o):
        return self.v != self._val(o)

    def __float__(self):
        return self.v

    def __repr__(self):
        return f"F32({self.v!r})"

    __hash__ = None


def _div(a: float, b: float) -> float:
    if b == 0.0:
        if a == 0.0 or a != a:
            return float("nan")
        return _math.copysign(float("inf"), a) * _math.copysign(1.0, b)
    return a / b


def float32(x):
    """``numba.float32`` used as a cast."""
    return F32(_r32(float(x)))


class _MathShim:
    pi = _math.pi

    @staticmethod
    def _f(fn, x):
        if isinstance(x, F32):
            return F32(_r32(fn(x.v)))
        return fn(float(x))

    @classmethod
    def sqrt(cls, x):
        return cls._f(_math.sqrt, x)

    @classmethod
    def tan(cls, x):
        return cls._f(_math.tan, x)

    @classmethod
    def acos(cls, x):
        return cls._f(_math.acos, x)

    @classmethod
    def tanh(cls, x):
        return cls._f(_math.tanh, x)


def _nb_max(a, b):
    r = a if a >= b else b
    if isinstance(a, F32) and isinstance(b, F32):
        return r
    return float(r)


class _LocalF32Array:
    def __init__(self, n):
        self._v = [0.0] * int(n)

    def __getitem__(self, i):
        return F32(self._v[i])

    def __setitem__(self, i, val):
        self._v[i] = _r32(float(val))


class TypedArray:
    """Wraps a NumPy array so that element reads carry Numba's scalar type."""

    def __init__(self, arr: np.ndarray, read_as_f64: bool = False):
        self.a = arr
        self.is_f32 = arr.dtype == np.float32 and not read_as_f64
        self.is_float = arr.dtype.kind == "f"
        self.shape = arr.shape

    def __getitem__(self, idx):
        v = self.a[idx]
        if self.is_f32:
            return F32(float(v))
        if self.is_float:
            return float(v)
        return int(v)

    def __setitem__(self, idx, val):
        if self.is_float:
            self.a[idx] = float(val)
        else:
            self.a[idx] = int(val)


class _Atomic:
    @staticmethod
    def max(arr, idx, val):
        old = arr[idx]
        arr[idx] = max(int(old), int(val))
        return old


class _Local:
    @staticmethod
    def array(n, dtype):
        assert dtype is float32, "only float32 local arrays are used by the reference kernels"
        return _LocalF32Array(n)


class _Kernel:
    def __init__(self, fn):
        self.fn = fn

    def __getitem__(self, cfg):
        blocks, threads = cfg
        blocks = tuple(blocks) if isinstance(blocks, (tuple, list)) else (blocks,)
        threads = tuple(threads) if isinstance(threads, (tuple, list)) else (threads,)

        def launch(*args):
            ranges = [range(b * t) for b, t in zip(blocks, threads)]
            for gid in itertools.product(*ranges):
                _CUDA.current = gid
                self.fn(*args)

        return launch


class _CudaModule(types.ModuleType):
    current = (0, 0, 0)
    atomic = _Atomic
    local = _Local

    def grid(self, ndim):
        return self.current[:ndim] if ndim > 1 else self.current[0]

    def jit(self, fn=None, device=False, inline=False, **_):
        def wrap(f):
            return f if device else _Kernel(f)

        if fn is None:
            return wrap
        return wrap(fn)


_CUDA = _CudaModule("numba.cuda")


def install() -> None:
    """Register the fake ``numba`` / ``numba.cuda`` modules."""
    nb = types.ModuleType("numba")
    nb.cuda = _CUDA
    nb.float32 = float32
    nb.int32 = int
    sys.modules["numba"] = nb
    sys.modules["numba.cuda"] = _CUDA


def load_reference_kernels(path: str, name: str = "reference_gpu_kernels_3d"):
    """Execute a reference kernel module (3D or 2D) under the shim and return it."""
    install()
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.math = _MathShim
    mod.max = _nb_max
    return mod


def scalar(x, is_f32: bool):
    """A kernel scalar argument typed as the caller's NumPy scalar would be."""
    return F32(_r32(float(x))) if is_f32 else float(x)
