"""Test-only stand-in for the one part of numba the reference's verification
harness uses: ``numba.cuda`` device arrays and synchronisation, backed by
torch CUDA tensors.  The kernels themselves come from this library's drop-in
module ``src/gpu_kernels_3d.py``; nothing here compiles or runs kernels."""

from . import cuda  # noqa: F401
