"""The plain-method FP64 configuration exactly, on both GPU tiers, against
the CPU oracle:

  32 x 32 x 32 cells, periodic x, y and clamped ("mirror") z; liquid = phase 0;
  8 grains from the Voronoi cells of 8 seed points drawn uniformly in the
  bottom 8 z-layers, each with a uniform-random unit quaternion; tanh front
  of the config_3d.yaml width at z = 8; temperature from the config gradient
  with uniform cooling; anisotropy and torque on; config_3d.yaml physics;
  KMAX = 50; 10 steps.

Tolerances:
  dense drop-in tier, FP64 (float64 phi, temperature and scalars): phi within
    1e-12 of the oracle after every step, nf and the valid part of mf equal,
    temperature equal;
  dense drop-in tier, the reference's production typing (float32 phi and
    scalars): phi within 1e-6, nf and mf equal;
  compact FP32 tier: max|dphi| <= 1e-4 against the FP64 oracle, sum to one
    within 1e-5, and the active-phase counts of the final state equal the
    oracle's APT of its final state.

The batched bicrystal engine is held to the same FP32 bar against the FP64
oracle run of each instance on its own.
"""
import numpy as np
import pytest

import oracle as O
from _helpers import valid_mf_equal

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

SEED, ORIENT_SEED = 2026, 7
STEPS = 10
TOL_F64, TOL_F32_TYPING, TOL_FP32 = 1e-12, 1e-6, 1e-4


def c1_case(dtype):
    from mpf3d import inputs
    return inputs.voronoi_case(32, 32, 32, 8, 8, seed=SEED, orientation_seed=ORIENT_SEED, dtype=dtype)


def oracle_history(case, f64):
    dt = np.float64 if f64 else np.float32
    sc = O.make_scalars([float(v) for v in case.phys.kernel_scalars(f32=not f64)], not f64)
    rate = case.phys.derived()["cooling_rate"]
    _, _, _, _, hist = O.run(case.phi.astype(dt), case.temp.astype(dt), case.wij, case.aij, case.mij, case.n111,
                             sc, STEPS, cooling_rate=rate, rate_f32=not f64, checked=True, switchable=True,
                             aniso=1, torque=1, record=True)
    return hist


def gpu_dense_history(case, f64):
    from src import gpu_kernels_3d as K
    dt = np.float64 if f64 else np.float32
    N, nx, ny, nz = case.phi.shape
    dev = torch.device("cuda:0")
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    p, q = t(case.phi.astype(dt)), t(case.phi.astype(dt))
    T = t(case.temp.astype(dt))
    mf = torch.zeros((K.KMAX, nx, ny, nz), dtype=torch.int32, device=dev)
    nf = torch.zeros((nx, ny, nz), dtype=torch.int32, device=dev)
    st = torch.zeros(2, dtype=torch.int32, device=dev)
    W, A, M, U = t(case.wij), t(case.aij), t(case.mij), t(case.n111)
    sc = case.phys.kernel_scalars(f32=not f64)
    rate = dt(case.phys.derived()["cooling_rate"])
    cfg = ((8, 8, 8), (4, 4, 4))
    hist = []
    for _ in range(STEPS):
        K.kernel_update_temp_3d[cfg](T, rate, nx, ny, nz)
        K.kernel_update_nfmf_3d_checked[cfg](p, mf, nf, st, nx, ny, nz, N)
        K.kernel_update_phasefield_active_3d_switchable[cfg](p, q, T, mf, nf, W, A, M, U, nx, ny, nz, N, *sc,
                                                             np.int32(1), np.int32(1))
        p, q = q, p
        hist.append((p.cpu().numpy(), nf.cpu().numpy(), mf.cpu().numpy(), st.cpu().numpy(), T.cpu().numpy()))
    K.check_errors()
    return hist


@pytest.mark.parametrize("f64", [True, False], ids=["fp64", "f32_typing"])
def test_c1_dense_tier_matches_oracle_every_step(f64):
    case = c1_case(np.float64 if f64 else np.float32)
    assert case.phi.shape == (9, 32, 32, 32)
    want = oracle_history(case, f64)
    got = gpu_dense_history(case, f64)
    tol = TOL_F64 if f64 else TOL_F32_TYPING
    for s, ((gp, gnf, gmf, gst, gT), (wp, wnf, wmf, wst, wT)) in enumerate(zip(got, want), 1):
        assert np.array_equal(gnf, wnf), f"step {s}: nf differs"
        assert valid_mf_equal(gmf, wmf, wnf), f"step {s}: mf differs"
        assert np.array_equal(gst, wst) and gst[0] == 0, f"step {s}: status {gst.tolist()} vs {wst.tolist()}"
        assert np.array_equal(gT, wT), f"step {s}: temperature differs"
        err = float(np.abs(gp.astype(np.float64) - wp.astype(np.float64)).max())
        assert err <= tol, f"step {s}: max|dphi| = {err:.3e}"
    # the run is not trivial: the front moved and junctions hold several phases
    assert int(want[-1][1].max()) >= 3
    assert float(np.abs(want[-1][0] - case.phi).max()) > 1e-3


def test_c1_compact_fp32_matches_fp64_oracle():
    from mpf3d.solver import CompactSolver
    case = c1_case(np.float64)
    want = oracle_history(case, True)
    ref = want[-1][0]
    s = CompactSolver(case.phi, case.temp, case.n111, case.wij, case.aij, case.mij, case.phys, slots=8)
    errs = []
    for k in range(STEPS):
        s.step(1)
        errs.append(float(np.abs(s.to_dense(np.float64) - want[k][0]).max()))
    assert max(errs) <= TOL_FP32, f"max|dphi| per step: {errs}"
    got = s.to_dense(np.float64)
    assert np.abs(got.sum(axis=0) - 1.0).max() < 1e-5
    mf = np.zeros((50,) + ref.shape[1:], np.int32)
    nf = np.zeros(ref.shape[1:], np.int32)
    O.apt(np.ascontiguousarray(ref), mf, nf, np.zeros(2, np.int32))
    assert np.array_equal(s.active_count(), nf)


def test_batched_engine_matches_fp64_oracle_per_instance():
    """Each instance of a batched step against the FP64 oracle run of that
    instance alone: its initial field, its undercooling (uniform temperature,
    no cooling), its anisotropy strength and orientation pair."""
    from mpf3d import inputs
    from mpf3d.batched import BatchedBicrystals
    dims = [(32, 16, 24), (24, 8, 20), (40, 12, 16)]
    dT, da = [1.25, 2.5, 0.5], [0.25, 0.5, 0.75]
    rng = np.random.default_rng(5)
    q = rng.standard_normal((len(dims), 2, 4))
    q /= np.linalg.norm(q, axis=2, keepdims=True)
    b = BatchedBicrystals(dims, q, dT, da, base_height=8.0, slots=4)
    init = [b.dense(i).astype(np.float64) for i in range(len(dims))]
    steps = 6
    b.step(steps, use_graph=False)
    b.check()
    for i, (nx, ny, nz) in enumerate(dims):
        phys = inputs.Physics(delta_a=da[i])
        n111 = inputs.rotated_n111(np.array([[0, 0, 0, 1.0], q[i, 0], q[i, 1]]))
        wij, aij, mij = inputs.matrices_for(phys, 3)
        temp = np.full((nx, ny, nz), phys.T_melt - dT[i], np.float64)
        sc = O.make_scalars([float(v) for v in phys.kernel_scalars(f32=False)], False)
        ref, _, _, _ = O.run(init[i], temp, wij, aij, mij, n111, sc, steps, cooling=False, switchable=True,
                             aniso=1, torque=1)
        err = float(np.abs(b.dense(i).astype(np.float64) - ref).max())
        assert err <= TOL_FP32, f"instance {i}: max|dphi| = {err:.3e}"
        assert float(np.abs(ref - init[i]).max()) > 1e-4  # the instance evolved
