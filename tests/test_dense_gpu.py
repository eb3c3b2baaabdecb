"""Dense drop-in tier on the GPU (through src/gpu_kernels_3d.py -> C ABI ->
sm_103a kernels) against the golden vectors of the reference's own kernel
source and against the oracle.

Tolerances: float64 phi within 1e-12 (last-bit differences of CUDA versus
host libm transcendentals), float32 phi within 1e-6; nf, mf, status and the
temperature field exact."""
import numpy as np
import pytest

import oracle as O
from _helpers import golden_files, golden_id, valid_mf_equal

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

TOL = {np.dtype(np.float64): 1e-12, np.dtype(np.float32): 1e-6}


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda:0")


def run_dropin(phi0, temp0, wij, aij, mij, n111, scalars, steps, rate, *, checked, switchable,
               aniso=1, torque=1, cooling=True, stream=None):
    from src import gpu_kernels_3d as K
    N, nx, ny, nz = phi0.shape
    phi, phi_new, temp = dev(phi0), dev(phi0.copy()), dev(temp0)
    mf = torch.zeros((max(50, N), nx, ny, nz), dtype=torch.int32, device="cuda:0")
    nf = torch.zeros((nx, ny, nz), dtype=torch.int32, device="cuda:0")
    st = torch.zeros(2, dtype=torch.int32, device="cuda:0")
    W, A, M, U = dev(wij), dev(aij), dev(mij), dev(n111)
    cfg = ((1, 1, 1), (4, 4, 4)) if stream is None else ((1, 1, 1), (4, 4, 4), stream)
    hist = []
    for _ in range(steps):
        if cooling:
            K.kernel_update_temp_3d[cfg](temp, rate, nx, ny, nz)
        st.zero_()
        if checked:
            K.kernel_update_nfmf_3d_checked[cfg](phi, mf, nf, st, nx, ny, nz, N)
        else:
            K.kernel_update_nfmf_3d[cfg](phi, mf, nf, nx, ny, nz, N)
        args = (phi, phi_new, temp, mf, nf, W, A, M, U, nx, ny, nz, N) + tuple(scalars)
        if switchable:
            K.kernel_update_phasefield_active_3d_switchable[cfg](*args, np.int32(aniso), np.int32(torque))
        else:
            K.kernel_update_phasefield_active_3d[cfg](*args)
        phi, phi_new = phi_new, phi
        torch.cuda.synchronize()
        hist.append((phi.cpu().numpy(), nf.cpu().numpy(), mf.cpu().numpy(), st.cpu().numpy(),
                     temp.cpu().numpy()))
    K.check_errors()
    return hist


@pytest.mark.parametrize("path", golden_files("run"), ids=golden_id)
def test_dropin_matches_reference_golden(path):
    g = np.load(path)
    f32 = bool(g["scalars_f32"])
    cast = np.float32 if f32 else np.float64
    sc = tuple(cast(v) for v in g["scalars"])
    hist = run_dropin(g["phi0"], g["temp0"], g["wij"], g["aij"], g["mij"], g["n111"], sc,
                      int(g["steps"]), cast(g["cooling_rate"]), checked=bool(g["checked"]),
                      switchable=str(g["kernel"]) == "switchable", aniso=int(g["aniso"]),
                      torque=int(g["torque"]), cooling=bool(g["cooling"]))
    tol = TOL[g["phi0"].dtype]
    for s, (p, n, m, st, t) in enumerate(hist):
        assert np.array_equal(n, g["nf"][s]), f"nf differs at step {s}"
        assert valid_mf_equal(m, g["mf"][s], n), f"mf differs at step {s}"
        if bool(g["checked"]):
            assert np.array_equal(st, g["status"][s])
        assert np.array_equal(t, g["temp"][s]), f"temperature differs at step {s}"
        err = np.abs(p.astype(np.float64) - g["phi"][s].astype(np.float64)).max()
        assert err <= tol, f"step {s}: max|dphi| = {err:.3e} > {tol}"


@pytest.mark.parametrize("phi_dtype", [np.float32, np.float64])
def test_dropin_matches_oracle_voronoi(phi_dtype):
    from mpf3d import inputs
    case = inputs.voronoi_case(24, 20, 28, 8, 8, seed=11, orientation_seed=12, undercooling=3.0)
    f32 = phi_dtype == np.float32
    sc = case.phys.kernel_scalars(f32=f32)
    phi0 = case.phi.astype(phi_dtype)
    temp0 = case.temp.astype(phi_dtype)
    rate = (np.float32 if f32 else np.float64)(case.phys.derived()["cooling_rate"])
    steps = 4
    hist = run_dropin(phi0, temp0, case.wij, case.aij, case.mij, case.n111, sc, steps, rate,
                      checked=True, switchable=True)
    osc = O.make_scalars([float(v) for v in sc], f32)
    _, _, _, _, ohist = O.run(phi0, temp0, case.wij, case.aij, case.mij, case.n111, osc, steps,
                              cooling_rate=float(rate), rate_f32=f32, record=True)
    tol = TOL[np.dtype(phi_dtype)]
    for s in range(steps):
        p, n, m, st, t = hist[s]
        op, on, om, ost, ot = ohist[s]
        assert np.array_equal(n, on) and valid_mf_equal(m, om, n)
        assert np.array_equal(st, ost)
        err = np.abs(p.astype(np.float64) - op.astype(np.float64)).max()
        assert err <= tol, f"step {s}: {err:.3e}"


def test_dropin_on_side_stream():
    g = np.load(golden_files("run")[0])
    f32 = bool(g["scalars_f32"])
    cast = np.float32 if f32 else np.float64
    sc = tuple(cast(v) for v in g["scalars"])
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        hist = run_dropin(g["phi0"], g["temp0"], g["wij"], g["aij"], g["mij"], g["n111"], sc, 2,
                          cast(g["cooling_rate"]), checked=bool(g["checked"]),
                          switchable=str(g["kernel"]) == "switchable", aniso=int(g["aniso"]),
                          torque=int(g["torque"]), stream=s.cuda_stream)
    tol = TOL[g["phi0"].dtype]
    for k in range(2):
        assert np.abs(hist[k][0].astype(np.float64) - g["phi"][k]).max() <= tol


def test_apt_known_answers_on_gpu():
    from src import gpu_kernels_3d as K
    for path in golden_files("apt"):
        g = np.load(path)
        phi = dev(g["phi0"])
        N, nx, ny, nz = g["phi0"].shape
        mf = torch.zeros((max(50, N), nx, ny, nz), dtype=torch.int32, device="cuda:0")
        nf = torch.zeros((nx, ny, nz), dtype=torch.int32, device="cuda:0")
        st = torch.zeros(2, dtype=torch.int32, device="cuda:0")
        K.kernel_update_nfmf_3d_checked[(1, 1, 1), (4, 4, 4)](phi, mf, nf, st, nx, ny, nz, N)
        torch.cuda.synchronize()
        assert np.array_equal(st.cpu().numpy(), g["status"])
        assert np.array_equal(nf.cpu().numpy(), g["nf"])
        assert valid_mf_equal(mf.cpu().numpy(), g["mf"], g["nf"])


def test_device_errors_are_reported_not_run_past():
    """nf above KMAX in the update and an unchecked APT deeper than mf are
    recorded in the error word; the kernels stay in bounds."""
    from src import gpu_kernels_3d as K
    from mpf3d import inputs
    case = inputs.voronoi_case(8, 8, 8, 2, 3, seed=1)
    N, nx, ny, nz = case.phi.shape
    phi, phi_new, temp = dev(case.phi), dev(case.phi.copy()), dev(case.temp)
    mf = torch.zeros((50, nx, ny, nz), dtype=torch.int32, device="cuda:0")
    nf = torch.zeros((nx, ny, nz), dtype=torch.int32, device="cuda:0")
    nf[1, 1, 1] = 60
    sc = case.phys.kernel_scalars()
    K.kernel_update_phasefield_active_3d[(1, 1, 1), (4, 4, 4)](
        phi, phi_new, temp, mf, nf, dev(case.wij), dev(case.aij), dev(case.mij), dev(case.n111),
        nx, ny, nz, N, *sc)
    with pytest.raises(RuntimeError, match="KMAX"):
        K.check_errors()
    shallow = torch.zeros((1, nx, ny, nz), dtype=torch.int32, device="cuda:0")
    K.kernel_update_nfmf_3d[(1, 1, 1), (4, 4, 4)](phi, shallow, nf, nx, ny, nz, N)
    with pytest.raises(RuntimeError, match="depth|rows"):
        K.check_errors()
    K.check_errors()
