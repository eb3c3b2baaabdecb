"""The remaining verification cases of the reference's 3D suite
(tests/verification_cases.py) on GB300:
  * through the drop-in kernels, driven the way the reference's harness
    drives them (run_3d_simulation, tests/verification_3d.py:771-936): the
    reference's pass rule, and the values the reference recorded on its own
    GPU run (tests/verification_report.md) to 1e-9 relative;
  * through the compact FP32 tier: the pass rule."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
pytest.importorskip("scipy")
import verification_cases as V
from mpf3d import inputs


def dropin_runner(phi0, temp_value, quats, phys, steps, aniso, torque, sample_every=None, observer=None):
    from src import gpu_kernels_3d as K
    N, nx, ny, nz = phi0.shape
    dev = "cuda:0"
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    phi, phi_new = t(phi0.astype(np.float32)), t(phi0.astype(np.float32))
    temp = t(np.full((nx, ny, nz), np.float32(temp_value), np.float32))
    mf = torch.zeros((50, nx, ny, nz), dtype=torch.int32, device=dev)
    nf = torch.zeros((nx, ny, nz), dtype=torch.int32, device=dev)
    st = torch.zeros(2, dtype=torch.int32, device=dev)
    wij, aij, mij = inputs.matrices_for(phys, N)
    W, A, M, U = t(wij), t(aij), t(mij), t(inputs.rotated_n111(quats))
    sc = phys.kernel_scalars(f32=True)
    rate = np.float32(phys.derived()["cooling_rate"])
    cfg = ((-(-nx // 4), -(-ny // 4), -(-nz // 4)), (4, 4, 4))
    samples = []
    for step in range(1, steps + 1):
        if float(rate) != 0.0:
            K.kernel_update_temp_3d[cfg](temp, rate, nx, ny, nz)
        st.zero_()
        K.kernel_update_nfmf_3d_checked[cfg](phi, mf, nf, st, nx, ny, nz, N)
        assert int(st[0]) == 0
        K.kernel_update_phasefield_active_3d_switchable[cfg](phi, phi_new, temp, mf, nf, W, A, M, U, nx, ny, nz, N,
                                                             *sc, np.int32(aniso), np.int32(torque))
        phi, phi_new = phi_new, phi
        if observer is not None and (step % sample_every == 0 or step == steps):
            samples.append(observer(phi.cpu().numpy(), step))
    torch.cuda.synchronize()
    K.check_errors()
    return phi.cpu().numpy(), samples


def compact_runner(phi0, temp_value, quats, phys, steps, aniso, torque, sample_every=None, observer=None):
    from mpf3d.solver import CompactSolver
    N, nx, ny, nz = phi0.shape
    wij, aij, mij = inputs.matrices_for(phys, N)
    s = CompactSolver(phi0, np.full(nz, temp_value), inputs.rotated_n111(quats), wij, aij, mij, phys,
                      anisotropy=bool(aniso), torque=bool(torque))
    samples, done = [], 0
    chunk = sample_every or steps
    while done < steps:
        k = min(chunk, steps - done)
        s.step(k)
        done += k
        if observer is not None:
            samples.append(observer(s.to_dense(np.float32), done))
    return s.to_dense(np.float32), samples


@pytest.fixture(scope="module")
def scan_cache():
    return {}


@pytest.mark.parametrize("name", list(V.CASES))
def test_dropin_case_matches_recorded_reference_run(name, scan_cache):
    vals, passed = V.run_case(name, dropin_runner, cache=scan_cache)
    assert passed, vals
    assert V.compare_recorded(name, vals) == []


@pytest.mark.parametrize("name", list(V.CASES))
def test_compact_case_passes(name, scan_cache):
    vals, passed = V.run_case(name, compact_runner, cache=scan_cache)
    assert passed, vals
