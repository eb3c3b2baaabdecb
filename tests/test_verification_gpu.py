"""Physics verification cases of the reference's 3D suite, restated: same
set-ups and pass rules as tests/verification_3d.py (basic_constraints
:1433-1456, static_flat_interface :1483-1506, isotropic_orientation_independence
:1568-1594, anisotropic_preferred_growth :1597-1634, torque_term_contribution
:1637-1660, grain_competition :1663-1693), run through the drop-in kernels the
way its harness runs them (run_3d_simulation :771-936: temperature kernel,
checked APT, switchable update, float32 arrays and scalars), and the simpler
ones also through the compact FP32 tier."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
Rotation = pytest.importorskip("scipy.spatial.transform").Rotation

DX = 1.0e-4


def quats_of(*rotations):
    q = np.zeros((len(rotations) + 1, 4))
    q[0] = (0, 0, 0, 1)
    for i, r in enumerate(rotations, 1):
        q[i] = r.as_quat()
    return q


def align_111_to_z():
    rot, _ = Rotation.align_vectors(np.array([[0.0, 0.0, 1.0]]), np.array([[1.0, 1.0, 1.0]]) / math.sqrt(3.0))
    return rot


def run_dropin(phi0, temp_value, quats, phys, steps, aniso, torque):
    from mpf3d import inputs
    from src import gpu_kernels_3d as K
    N, nx, ny, nz = phi0.shape
    dev = "cuda:0"
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    phi, phi_new = t(phi0), t(phi0.copy())
    temp = t(np.full((nx, ny, nz), np.float32(temp_value), np.float32))
    mf = torch.zeros((50, nx, ny, nz), dtype=torch.int32, device=dev)
    nf = torch.zeros((nx, ny, nz), dtype=torch.int32, device=dev)
    st = torch.zeros(2, dtype=torch.int32, device=dev)
    wij, aij, mij = inputs.matrices_for(phys, N)
    W, A, M, U = t(wij), t(aij), t(mij), t(inputs.rotated_n111(quats))
    sc = phys.kernel_scalars(f32=True)
    rate = np.float32(phys.derived()["cooling_rate"])
    cfg = ((1, 1, 1), (4, 4, 4))
    nf_max = 0
    for _ in range(steps):
        if float(rate) != 0.0:
            K.kernel_update_temp_3d[cfg](temp, rate, nx, ny, nz)
        st.zero_()
        K.kernel_update_nfmf_3d_checked[cfg](phi, mf, nf, st, nx, ny, nz, N)
        torch.cuda.synchronize()
        assert int(st[0]) == 0
        nf_max = max(nf_max, int(st[1]))
        K.kernel_update_phasefield_active_3d_switchable[cfg](phi, phi_new, temp, mf, nf, W, A, M, U, nx, ny, nz, N,
                                                             *sc, np.int32(aniso), np.int32(torque))
        phi, phi_new = phi_new, phi
    torch.cuda.synchronize()
    K.check_errors()
    return phi.cpu().numpy().astype(np.float64), nf_max


def run_compact(phi0, temp_value, quats, phys, steps, aniso, torque):
    from mpf3d import inputs
    from mpf3d.solver import CompactSolver
    N, nx, ny, nz = phi0.shape
    wij, aij, mij = inputs.matrices_for(phys, N)
    s = CompactSolver(phi0, np.full(nz, temp_value), inputs.rotated_n111(quats), wij, aij, mij, phys,
                      anisotropy=bool(aniso), torque=bool(torque))
    s.step(steps)
    return s.to_dense(np.float64), int(s.active_count().max())


RUNNERS = {"dropin": run_dropin, "compact": run_compact}


def front(phi):
    """Per column: highest z with solid fraction > 0.5 (nan if none)."""
    mask = (1.0 - phi[0]) > 0.5
    nz = mask.shape[2]
    pos = np.where(mask.any(axis=2), nz - 1 - np.argmax(mask[:, :, ::-1], axis=2), np.nan)
    fin = pos[np.isfinite(pos)]
    return float(np.mean(fin) * DX), float(np.std(fin) * DX)


@pytest.mark.parametrize("runner", ["dropin", "compact"])
def test_basic_constraints(runner):
    from mpf3d import inputs
    phys = inputs.Physics()
    d = phys.derived()
    gmap = inputs.grain_map_2d(12, 8, 4, 17)
    phi0 = inputs.phi_from_grain_map_2d(gmap, 4, 14, DX, d["delta"], 4)
    q = inputs.random_quaternions(4, 23)
    phi, nf_max = RUNNERS[runner](phi0, phys.T_melt - 5.0, q, phys, 6, 1, 1)
    assert not np.isnan(phi).any()
    assert phi.min() >= -1e-5 and phi.max() <= 1 + 1e-5
    assert np.abs(phi.sum(axis=0) - 1.0).max() <= 5e-4
    assert nf_max <= 50


@pytest.mark.parametrize("runner", ["dropin", "compact"])
def test_static_flat_interface(runner):
    from mpf3d import inputs
    phys = inputs.Physics()
    d = phys.derived()
    phi0 = inputs.wavy_front(12, 6, 14, DX, d["delta"], 5, 0.0)
    q = quats_of(Rotation.identity())
    phi, _ = RUNNERS[runner](phi0, phys.T_melt, q, phys, 6, 0, 0)
    m0, _ = front(phi0.astype(np.float64))
    m1, rough = front(phi)
    assert abs(m1 - m0) <= 1.05 * DX
    assert rough <= 0.15 * DX


@pytest.mark.parametrize("runner", ["dropin", "compact"])
def test_isotropic_orientation_independence(runner):
    from mpf3d import inputs
    phys = inputs.Physics(delta_a=0.0, ksi=1.0)
    d = phys.derived()
    phi0 = inputs.wavy_front(12, 6, 14, DX, d["delta"], 5, 0.0)
    a, _ = RUNNERS[runner](phi0, phys.T_melt - 6.0, quats_of(Rotation.identity()), phys, 6, 0, 0)
    b, _ = RUNNERS[runner](phi0, phys.T_melt - 6.0, quats_of(align_111_to_z()), phys, 6, 0, 0)
    assert abs(front(a)[0] - front(b)[0]) <= 0.15 * DX
    assert abs(np.mean(1 - a[0]) - np.mean(1 - b[0])) <= 2e-4
    assert np.sqrt(np.mean((a[1] - b[1]) ** 2)) <= 2e-3


def test_anisotropic_preferred_growth():
    from mpf3d import inputs
    phys = inputs.Physics(delta_a=0.55, p_round=0.02)
    d = phys.derived()
    phi0 = inputs.wavy_front(16, 6, 18, DX, d["delta"], 6.0, 2.0, 0.2)
    a, _ = run_dropin(phi0, phys.T_melt, quats_of(Rotation.identity()), phys, 12, 1, 0)
    b, _ = run_dropin(phi0, phys.T_melt, quats_of(align_111_to_z()), phys, 12, 1, 0)
    (ma, ra), (mb, rb) = front(a), front(b)
    l2 = np.sqrt(np.mean((a[1] - b[1]) ** 2))
    assert abs(ma - mb) >= 0.10 * DX or abs(ra - rb) >= 0.05 * DX or l2 >= 5e-5


def test_torque_term_contribution():
    from mpf3d import inputs
    phys = inputs.Physics(delta_a=0.55, p_round=0.02)
    d = phys.derived()
    phi0 = inputs.wavy_front(16, 6, 18, DX, d["delta"], 6.0, 2.0, 0.3)
    q = quats_of(Rotation.from_euler("xyz", [20.0, 35.0, 10.0], degrees=True))
    off, _ = run_dropin(phi0, phys.T_melt, q, phys, 12, 1, 0)
    on, _ = run_dropin(phi0, phys.T_melt, q, phys, 12, 1, 1)
    l2 = np.sqrt(np.mean((on[1] - off[1]) ** 2))
    assert l2 >= 5e-5 or abs(front(on)[1] - front(off)[1]) >= 0.05 * DX


def test_grain_competition():
    from mpf3d import inputs
    phys = inputs.Physics()
    d = phys.derived()
    gmap = inputs.grain_map_2d(12, 12, 6, 31)
    phi0 = inputs.phi_from_grain_map_2d(gmap, 6, 16, DX, d["delta"], 5)
    q = inputs.random_quaternions(6, 11)
    phi, _ = run_dropin(phi0, phys.T_melt - 5.0, q, phys, 8, 1, 1)
    v0 = np.array([phi0[g].astype(np.float64).sum() * DX ** 3 for g in range(1, 7)])
    v1 = np.array([phi[g].sum() * DX ** 3 for g in range(1, 7)])
    assert (v1 > DX ** 3).sum() <= (v0 > DX ** 3).sum()
    assert np.abs(v1 - v0).max() >= 2e-14
