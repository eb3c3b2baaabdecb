"""FP32 compact tier against the FP64 drop-in tier where FP32 is most
exposed: a bicrystal growing with one grain's {111} facet along the front
normal (aligned_111_to_z | identity), strong kinetic anisotropy (ksi 0.01)
and 6 K undercooling -- the kinetic-regime set-up of the reference's
verification suite (tests/verification_3d.py:2326-2385).  Near the facet the
kinetic factor b(theta) is steep in theta, and theta must come out of a best
|cos| close to 1 without the cancellation of FP32 acos."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
pytest.importorskip("scipy")

TOL_PHI = 1e-4      # max |dphi| of FP32 against FP64 after 10 steps
TOL_ANGLE = 1e-3    # groove dihedral-like angle, degrees


def fp64_run(phi0, temp_value, quats, phys, steps, aniso):
    from mpf3d import inputs
    from src import gpu_kernels_3d as K
    N, nx, ny, nz = phi0.shape
    dev = "cuda:0"
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    p, q = t(phi0.astype(np.float64)), t(phi0.astype(np.float64))
    T = t(np.full((nx, ny, nz), temp_value, np.float64))
    mf = torch.zeros((50, nx, ny, nz), dtype=torch.int32, device=dev)
    nf = torch.zeros((nx, ny, nz), dtype=torch.int32, device=dev)
    wij, aij, mij = inputs.matrices_for(phys, N)
    W, A, M, U = t(wij), t(aij), t(mij), t(inputs.rotated_n111(quats))
    sc = phys.kernel_scalars(f32=False)
    cfg = ((-(-nx // 4), -(-ny // 4), -(-nz // 4)), (4, 4, 4))
    for _ in range(steps):
        K.kernel_update_nfmf_3d[cfg](p, mf, nf, nx, ny, nz, N)
        K.kernel_update_phasefield_active_3d_switchable[cfg](p, q, T, mf, nf, W, A, M, U, nx, ny, nz, N, *sc,
                                                             np.int32(aniso), np.int32(0))
        p, q = q, p
    torch.cuda.synchronize()
    K.check_errors()
    return p.cpu().numpy()


@pytest.mark.parametrize("undercooling,ksi,delta_a", [(6.0, 0.01, 0.35), (3.0, 0.05, 0.5), (0.25, 0.05, 0.5)])
def test_near_facet_kinetics_match_fp64(undercooling, ksi, delta_a):
    from mpf3d import groove, inputs
    from mpf3d.solver import CompactSolver
    phys = inputs.Physics(delta_a=delta_a, ksi=ksi, p_round=0.02, G=0.0, V_pulling=0.0)
    nx, ny, nz, split, steps = 18, 6, 28, 9, 10
    phi0 = inputs.bicrystal_field(nx, ny, nz, phys.dx, phys.derived()["delta"], 7.0, split, waviness=0.8)
    lib = inputs.orientation_library()
    q = inputs.quaternions_of([lib["aligned_111_to_z"], lib["identity"]])
    T = phys.T_melt - undercooling
    ref = fp64_run(phi0, T, q, phys, steps, 1)
    wij, aij, mij = inputs.matrices_for(phys, 3)
    s = CompactSolver(phi0, np.full(nz, T), inputs.rotated_n111(q), wij, aij, mij, phys, anisotropy=True,
                      torque=False)
    s.step(steps)
    got = s.to_dense(np.float64)
    assert np.abs(got - ref).max() <= TOL_PHI
    g_ref = groove.groove_metrics(ref, root_x_guess=float(split))
    g_got = groove.groove_metrics(got.astype(np.float32), root_x_guess=float(split))
    assert abs(g_got["dihedral_angle_like_deg"] - g_ref["dihedral_angle_like_deg"]) <= TOL_ANGLE
    f_ref = groove.family_volumes(ref, [1], [2], phys.dx)
    f_got = groove.family_volumes(got, [1], [2], phys.dx)
    assert f_got["winner_family"] == f_ref["winner_family"]
    assert f_got["winner_loser_volume_ratio"] == pytest.approx(f_ref["winner_loser_volume_ratio"], rel=1e-6)
