"""libmpf3d.so loads and exports every function include/mpf3d.h declares;
the drop-in validates arguments before touching the GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

from mpf3d import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", f)).read()
            names += re.findall(r"^\s*(?:int|void|int64_t|double|const char \*)\s+(mpf[23]d_\w+)\s*\(", txt, re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def libso():
    if not os.path.exists(_lib.LIB_PATH):
        import build as b
        b.build()
    return ctypes.CDLL(_lib.LIB_PATH)


def test_library_exports_every_declared_symbol(libso):
    names = declared_functions()
    assert "mpf3d_dense_update" in names
    missing = [n for n in names if not hasattr(libso, n)]
    assert not missing, f"missing exports: {missing}"
    for n in _lib.exported_symbols():
        assert n in names, f"binding declares {n} that the header does not"


class FakeDev:
    def __init__(self, shape, dtype):
        self.__cuda_array_interface__ = {"shape": shape, "typestr": np.dtype(dtype).str,
                                         "data": (0x1000, False), "version": 3, "strides": None}


def test_dropin_rejects_bad_arguments():
    from src import gpu_kernels_3d as K
    phi = FakeDev((3, 4, 4, 4), np.float16)
    mf = FakeDev((50, 4, 4, 4), np.int32)
    nf = FakeDev((4, 4, 4), np.int32)
    with pytest.raises(TypeError):
        K.kernel_update_nfmf_3d[(1, 1, 1), (4, 4, 4)](phi, mf, nf, 4, 4, 4, 3)
    phi = FakeDev((3, 4, 4, 4), np.float32)
    with pytest.raises(ValueError):
        K.kernel_update_nfmf_3d[(1, 1, 1), (4, 4, 4)](phi, mf, nf, 4, 4, 5, 3)
    with pytest.raises(TypeError):
        K.kernel_update_nfmf_3d[(1, 1, 1), (4, 4, 4)](phi, FakeDev((50, 4, 4, 4), np.int64), nf, 4, 4, 4, 3)
    with pytest.raises(ValueError):
        K.kernel_update_nfmf_3d[(1, 1, 1), (4, 4, 4)](phi, FakeDev((50, 4, 4, 3), np.int32), nf, 4, 4, 4, 3)
    with pytest.raises(ValueError):  # Numba also raises ValueError without a launch config
        K.kernel_update_nfmf_3d(phi, mf, nf, 4, 4, 4, 3)
    with pytest.raises(TypeError):
        K.kernel_update_temp_3d[(1,), (1,)]([1.0], np.float32(1.0), 4, 4, 4)


def test_dropin_exports_reference_names():
    from src import gpu_kernels_3d as K
    assert K.KMAX == 50 and K.LIQ == 0
    for n in ("kernel_update_nfmf_3d", "kernel_update_nfmf_3d_checked",
              "kernel_update_phasefield_active_3d", "kernel_update_phasefield_active_3d_switchable",
              "kernel_update_temp_3d"):
        assert hasattr(K, n)
