"""Observables, slices, checkpoints and the batched orientation scan on the
GPU, each against a host restatement of the reference function it replaces
(compute_metrics_3d / interface_positions_3d, tests/verification_3d.py:
409-416, 612-654; numpy.argmax slices of src/plot_utils_3d.py:36-72;
init_singlemode_sphere_3d, src/seed_modes_3d.py:59-113; measure_observables,
run_orientation_scan_3d.py:238-394) applied to the dense field of the same
state, and the scan against the dense drop-in path."""
import math

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def make_solver(case, **kw):
    from mpf3d.solver import CompactSolver
    return CompactSolver(case.phi, case.temp, case.n111, case.wij, case.aij, case.mij, case.phys, **kw)


# -- host restatements (checkers) ---------------------------------------------------------
def interface_positions_np(phi, threshold=0.5):
    solid = 1.0 - phi[0]
    mask = solid > threshold
    nz = mask.shape[2]
    has = mask.any(axis=2)
    rev = np.argmax(mask[:, :, ::-1], axis=2)
    return np.where(has, nz - 1 - rev, np.nan).astype(np.float64)


def metrics_np(phi, nf, dx):
    s = phi.astype(np.float64).sum(axis=0)
    gv = [float(phi[g].astype(np.float64).sum() * dx ** 3) for g in range(1, phi.shape[0])]
    pos = interface_positions_np(phi)
    fin = pos[np.isfinite(pos)]
    solid = (1.0 - phi[0]).astype(np.float64)
    return {"phi_sum_error_max": float(np.max(np.abs(s - 1.0))), "phi_min": float(phi.min()),
            "phi_max": float(phi.max()), "nf_max": int(nf.max()), "nan_count": int(np.isnan(phi).sum()),
            "solid_fraction": float(solid.mean()), "solid_volume": float(solid.sum() * dx ** 3),
            "grain_volumes": gv, "surviving_grains": int(sum(v > dx ** 3 for v in gv)),
            "interface_position_mean": float(fin.mean() * dx), "interface_position_max": float(fin.max() * dx),
            "interface_position_std": float(fin.std() * dx)}


def trilinear_np(f, x, y, z):
    nx, ny, nz = f.shape
    if x < 0 or y < 0 or z < 0 or x > nx - 1 or y > ny - 1 or z > nz - 1:
        return float("nan")
    x0, y0, z0 = int(math.floor(x)), int(math.floor(y)), int(math.floor(z))
    x1, y1, z1 = min(x0 + 1, nx - 1), min(y0 + 1, ny - 1), min(z0 + 1, nz - 1)
    tx, ty, tz = x - x0, y - y0, z - z0
    c00 = f[x0, y0, z0] * (1 - tx) + f[x1, y0, z0] * tx
    c01 = f[x0, y0, z1] * (1 - tx) + f[x1, y0, z1] * tx
    c10 = f[x0, y1, z0] * (1 - tx) + f[x1, y1, z0] * tx
    c11 = f[x0, y1, z1] * (1 - tx) + f[x1, y1, z1] * tx
    return float((c00 * (1 - ty) + c10 * ty) * (1 - tz) + (c01 * (1 - ty) + c11 * ty) * tz)


def radius_one_side_np(f, c, d, thr=0.5, step=0.5):
    d = np.asarray(d, np.float64)
    d = d / np.linalg.norm(d)
    up = np.array(f.shape, np.float64) - 1.0
    lims = [((u - ci) / di if di > 0 else -ci / di) for ci, di, u in zip(c, d, up) if abs(di) >= 1e-12]
    lims = [x for x in lims if x > 0]
    max_s = min(lims) if lims else 0.0
    if max_s <= 0:
        return float("nan")
    v0 = trilinear_np(f, *c)
    if not np.isfinite(v0) or v0 < thr:
        return float("nan")
    ps, pv = 0.0, v0
    for i in range(1, max(2, int(math.ceil(max_s / step)) + 1) + 1):
        s = min(i * step, max_s)
        v = trilinear_np(f, *(np.asarray(c) + d * s))
        if not np.isfinite(v):
            break
        if pv >= thr and v < thr:
            dv = pv - v
            if abs(dv) < 1e-12:
                return float(s)
            return float(ps + min(max((pv - thr) / dv, 0.0), 1.0) * (s - ps))
        ps, pv = s, v
    return float("nan")


def radius_np(f, c, d, step=0.5):
    v = [x for x in (radius_one_side_np(f, c, d, step=step), radius_one_side_np(f, c, -np.asarray(d), step=step))
         if np.isfinite(x)]
    return float(np.mean(v)) if v else float("nan")


def sphere_np(nx, ny, nz, dx, delta, radius_cells):
    factor = np.float32(2.2 / delta)
    X, Y, Z = np.meshgrid(np.arange(nx) * dx, np.arange(ny) * dx, np.arange(nz) * dx, indexing="ij")
    dist = np.sqrt((X - nx * dx / 2.0) ** 2 + (Y - ny * dx / 2.0) ** 2 + (Z - nz * dx / 2.0) ** 2)
    phs = (0.5 * (1.0 - np.tanh(factor * (dist - radius_cells * dx)))).astype(np.float32)
    return np.stack([1.0 - phs, phs]).astype(np.float32)


# -- tests -----------------------------------------------------------------------------------
def _stepped_case():
    from mpf3d import inputs
    case = inputs.voronoi_case(26, 18, 30, 7, 9, seed=4, orientation_seed=5)
    s = make_solver(case, slots=8)
    s.step(12)
    return case, s


def test_metrics_match_compute_metrics_on_the_dense_field():
    case, s = _stepped_case()
    phi = s.to_dense()
    nf = s.active_count()
    got = s.metrics()
    want = metrics_np(phi, nf, case.phys.dx)
    for k in ("nf_max", "nan_count", "surviving_grains"):
        assert got[k] == want[k], k
    for k in ("phi_min", "phi_max"):
        assert got[k] == want[k], k
    for k in ("phi_sum_error_max", "solid_fraction", "solid_volume", "interface_position_mean",
              "interface_position_max", "interface_position_std"):
        assert got[k] == pytest.approx(want[k], rel=1e-6, abs=1e-12), k
    assert np.allclose(got["grain_volumes"], want["grain_volumes"], rtol=1e-9, atol=0)
    pos = s.interface_positions()
    assert np.array_equal(np.isnan(pos), np.isnan(interface_positions_np(phi)))
    assert np.array_equal(np.nan_to_num(pos, nan=-1), np.nan_to_num(interface_positions_np(phi), nan=-1))


@pytest.mark.parametrize("axis", ["xy", "xz", "yz"])
def test_phase_slices_match_numpy_argmax(axis):
    _, s = _stepped_case()
    phi = s.to_dense()
    for index in (None, 0, 7):
        sl = s.phase_slice(axis, index)
        i = sl["index"]
        dense = {"xy": phi[:, :, :, i], "xz": phi[:, :, i, :], "yz": phi[:, i, :, :]}[axis]
        assert np.array_equal(sl["ids"], np.argmax(dense, axis=0))
        assert np.array_equal(sl["fraction"], dense.max(axis=0))
        assert np.array_equal(sl["solid"], (1.0 - dense[0]).astype(np.float32))


@pytest.mark.parametrize("load_slots", [None, 16])
def test_checkpoint_resume_is_exact(tmp_path, load_slots):
    from mpf3d.solver import CompactSolver
    case, s = _stepped_case()
    p = str(tmp_path / "ck.npz")
    info = s.save(p)
    assert info["entries"] > 0
    s.step(15)
    ref = s.to_dense()
    r = CompactSolver.load(p, slots=load_slots)
    assert r.step_count == 12 and r.slots == (load_slots or 8)
    r.step(15)
    assert np.array_equal(r.to_dense(), ref)
    assert r.metrics()["nf_max"] == s.metrics()["nf_max"]


def test_checkpoint_rejects_a_foreign_file(tmp_path):
    from mpf3d.solver import CompactSolver
    p = str(tmp_path / "x.npz")
    np.savez(p, format=np.array("something else"))
    with pytest.raises(ValueError):
        CompactSolver.load(p)


def test_sphere_init_and_ray_radii_match_the_reference_functions():
    from mpf3d import inputs
    from mpf3d.batched import BatchedBicrystals
    phys = inputs.Physics()
    d = phys.derived()
    dims = [(24, 20, 22), (17, 26, 19)]
    q = np.tile(np.array([0, 0, 0, 1.0]), (2, 2, 1))
    b = BatchedBicrystals(dims, q, [1.0, 1.0], [0.3, 0.3], phys, layout="sphere", radius=[6.0, 4.5])
    dirs = np.array([[1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 1, 1.0]])
    r = b.ray_radii(dirs)
    for i, (nx, ny, nz) in enumerate(dims):
        want = sphere_np(nx, ny, nz, phys.dx, d["delta"], [6.0, 4.5][i])
        got = b.dense(i)[:2]
        assert np.abs(got.astype(np.float64) - want).max() <= 6e-8  # float32 rounding of the same float64 value
        c = np.array([nx / 2.0, ny / 2.0, nz / 2.0])
        for j, dd in enumerate(dirs):
            assert r[i, j] == pytest.approx(radius_np(want[1].astype(np.float64), c, dd), abs=1e-6)


def test_orientation_scan_matches_the_dense_dropin_path():
    """Three cases of a reduced scan (28^3, radius 6, 0.2 K, 40 steps, samples
    every 10) on the batched FP32 engine against the reference's loop run
    through the dense drop-in kernels (unchecked APT, switchable update) in
    float64 -- phi and scalars, the accurate reference numerics -- with the
    observables measured on the host."""
    from mpf3d import inputs
    from mpf3d.scan import resolve_orientation_cases, run_orientation_scan, fit_growth_rate
    from src import gpu_kernels_3d as K
    phys = inputs.Physics()
    d = phys.derived()
    cases = resolve_orientation_cases()[:3]
    nx = ny = nz = 28
    dT = 0.2
    rep = run_orientation_scan(cases, dims=(nx, ny, nz), nsteps=40, save_every=10, radius_cells=6.0,
                               undercooling=dT, phys=phys)
    sc = phys.kernel_scalars(f32=False)
    wij, aij, mij = inputs.matrices_for(phys, 2)
    dev = "cuda:0"
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    c = np.array([nx / 2.0, ny / 2.0, nz / 2.0])
    for ci, case in enumerate(cases):
        q = np.array([[0, 0, 0, 1.0], case["quaternion"]])
        phi0 = sphere_np(nx, ny, nz, phys.dx, d["delta"], 6.0).astype(np.float64)
        p, pn = t(phi0), t(phi0.copy())
        temp = t(np.full((nx, ny, nz), phys.T_melt - dT, np.float64))
        mf = torch.zeros((20, nx, ny, nz), dtype=torch.int32, device=dev)
        nf = torch.zeros((nx, ny, nz), dtype=torch.int32, device=dev)
        W, A, M, U = t(wij), t(aij), t(mij), t(inputs.rotated_n111(q))
        rows = []
        for step in range(41):
            if step % 10 == 0:
                ph = p.cpu().numpy()
                vol = float(ph[1].astype(np.float64).sum() * phys.dx ** 3)
                rows.append({"time": step * phys.dt, "volume": vol,
                             "equivalent_radius": (3 * vol / (4 * math.pi)) ** (1 / 3),
                             "radius_x": radius_np(ph[1].astype(np.float64), c, [1, 0, 0]) * phys.dx,
                             "radius_diag111": radius_np(ph[1].astype(np.float64), c, [1, 1, 1]) * phys.dx})
            if step == 40:
                break
            cfg = ((7, 7, 7), (4, 4, 4))
            K.kernel_update_nfmf_3d[cfg](p, mf, nf, nx, ny, nz, 2)
            K.kernel_update_phasefield_active_3d_switchable[cfg](p, pn, temp, mf, nf, W, A, M, U, nx, ny, nz, 2,
                                                                 *sc, np.int32(1), np.int32(1))
            p, pn = pn, p
        K.check_errors()
        got = rep["timeseries"][case["label"]]
        assert len(got) == len(rows) == 5
        for g, w in zip(got, rows):
            # FP32 vs FP64 on this fast-growing case: the reference's own float32
            # kernels deviate from float64 by 7.4e-4 in volume after 40 steps
            assert g["volume"] == pytest.approx(w["volume"], rel=2e-3)
            assert g["radius_x"] == pytest.approx(w["radius_x"], abs=0.05 * phys.dx, nan_ok=True)
            assert g["radius_diag111"] == pytest.approx(w["radius_diag111"], abs=0.05 * phys.dx, nan_ok=True)
        assert np.isfinite(got[-1]["radius_x"]) and got[-1]["volume"] > got[0]["volume"]  # the grain grew
        rate = fit_growth_rate(rows, 0.5)[0]
        assert rep["summary"][ci]["fitted_growth_rate"] == pytest.approx(rate, rel=2e-2, abs=1e-9)
