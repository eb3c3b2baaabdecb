"""mpf3d_compact_step_noalloc: the compact step for hosts that cannot let a
library allocate device memory (a host that reserves the whole GPU memory
budget for its own pool, or a real-time loop that cannot afford a
synchronising cudaMalloc).  Its work list lives in a file-scope device array
of MPF3D_NOALLOC_MAX_CELLS entries instead of caller scratch.

Checked here through the C ABI against the existing entry point
(mpf3d_compact_step with caller scratch) on two calls in a row, within the
1e-6 tolerance of the exact-path tests (the same kernels run, so the results
are expected to be identical), and the size limit is checked to be refused.
This file sorts last so that a failure here does not stop the other tests.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

MAX_CELLS = 4194304
ERR_TOO_LARGE = -4


def _case():
    from mpf3d import inputs
    return inputs.voronoi_case(40, 32, 36, 8, 10, seed=21, orientation_seed=5, undercooling=2.5)


def _dense(lib, solver, bufs):
    out = torch.empty((solver.N, solver.nx, solver.ny, solver.nz), dtype=torch.float32, device="cuda:0")
    rc = lib.mpf3d_compact_to_dense(bufs[0].data_ptr(), bufs[1].data_ptr(), bufs[2].data_ptr(), solver.slots,
                                    solver.N, solver.nx, solver.ny, solver.nz, out.data_ptr(), 0, None)
    assert rc == 0
    return out.cpu().numpy()


def _noalloc_step(lib, s, src, dst, step_index):
    tmc = s.T_melt + step_index * s.cooling_rate
    return lib.mpf3d_compact_step_noalloc(
        src[0].data_ptr(), src[1].data_ptr(), src[2].data_ptr(), dst[0].data_ptr(), dst[1].data_ptr(),
        dst[2].data_ptr(), s.slots, s.amax, s.T0z.data_ptr(), tmc, s.wij.data_ptr(), s.a2ij.data_ptr(),
        s.mij.data_ptr(), s.n111.data_ptr(), s.N, s.nx, s.ny, s.nz, ctypes.byref(s.scalars),
        int(s.anisotropy), int(s.torque), int(s.symmetric_normals), s.err.data_ptr(), None)


def test_noalloc_step_matches_scratch_step_on_two_calls():
    from mpf3d import _lib
    from mpf3d.solver import CompactSolver
    lib = _lib.lib()
    case = _case()
    mk = lambda: CompactSolver(case.phi, case.temp, case.n111, case.wij, case.aij, case.mij, case.phys,
                               slots=8)
    ref = mk()
    ref.launch_step(1)
    ref_dense1 = ref.to_dense()
    ref.launch_step(2)
    ref_dense2 = ref.to_dense()
    ref.check()

    s = mk()
    a = s.buf[s.cur]
    b = s._alloc()
    c = s._alloc()
    assert _noalloc_step(lib, s, a, b, 1) == 0
    got1 = _dense(lib, s, b)
    assert _noalloc_step(lib, s, b, c, 2) == 0
    got2 = _dense(lib, s, c)
    torch.cuda.synchronize()
    assert int(s.err.item()) == 0
    assert np.abs(got1 - ref_dense1).max() <= 1e-6
    assert np.abs(got2 - ref_dense2).max() <= 1e-6
    assert np.array_equal((c[0] & 0x7F).cpu().numpy(), (ref.stored_counts()).cpu().numpy())


def test_noalloc_refuses_grids_above_its_array():
    from mpf3d import _lib
    lib = _lib.lib()
    t = torch.zeros(16, dtype=torch.int32, device="cuda:0")
    p = t.data_ptr()
    sc = _lib.Scalars()
    nx, ny, nz = 256, 256, 65  # 4,259,840 cells > 4,194,304
    assert nx * ny * nz > MAX_CELLS
    rc = lib.mpf3d_compact_step_noalloc(p, p, p, p, p, p, 8, 16, p, 0.0, p, p, p, p, 3, nx, ny, nz,
                                        ctypes.byref(sc), 1, 1, 1, p, None)
    assert rc == ERR_TOO_LARGE
