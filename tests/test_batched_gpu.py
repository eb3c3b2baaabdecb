"""Batched bicrystal engine on the GPU: one batched step equals stepping each
instance on its own (bit for bit), CUDA-graph replay equals eager launches,
and the GPU observables equal host reductions of the same states."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

DIMS = [(32, 16, 24), (64, 8, 20), (40, 24, 16)]
DT = [1.25, 2.5, 0.5]
DA = [0.25, 0.5, 0.75]


def make_batch(**kw):
    from mpf3d.batched import BatchedBicrystals
    rng = np.random.default_rng(3)
    q = rng.standard_normal((len(DIMS), 2, 4))
    q /= np.linalg.norm(q, axis=2, keepdims=True)
    return BatchedBicrystals(DIMS, q, DT, DA, base_height=8.0, **kw), q


def test_batched_step_equals_single_domain_runs():
    from mpf3d import inputs
    from mpf3d.solver import CompactSolver
    b, q = make_batch()
    init = [b.dense(i) for i in range(len(DIMS))]
    b.step(6, use_graph=False)
    b.check()
    for i, (nx, ny, nz) in enumerate(DIMS):
        phys = inputs.Physics(delta_a=DA[i])
        full_q = np.array([[0, 0, 0, 1.0], q[i, 0], q[i, 1]])
        n111 = inputs.rotated_n111(full_q)
        wij, aij, mij = inputs.matrices_for(phys, 3)
        temp = np.full(nz, phys.T_melt - DT[i])
        s = CompactSolver(init[i], temp, n111, wij, aij, mij, phys, cooling_rate=0.0, slots=4)
        s.step(6)
        single = s.to_dense()
        got = b.dense(i)
        assert np.array_equal(got, single), f"instance {i}: max diff {np.abs(got - single).max():.3e}"


def test_quiet_tiles_give_the_same_batch():
    """Skipping the quiet warp tiles of the batched sweep changes no bit of
    the batch, eager or from a CUDA graph, on ragged instances: x not a
    multiple of 32, y not a multiple of 8 (warps past the last row), z not a
    multiple of 4 and a one-tile-wide x."""
    from mpf3d.batched import BatchedBicrystals
    dims = [(33, 10, 17), (40, 24, 20), (24, 8, 26), (64, 16, 21)]
    rng = np.random.default_rng(5)
    q = rng.standard_normal((len(dims), 2, 4))
    q /= np.linalg.norm(q, axis=2, keepdims=True)
    dt, da = [0.75, 2.0, 1.5, 3.0], [0.2, 0.9, 0.5, 0.0]
    full = BatchedBicrystals(dims, q, dt, da, base_height=6.0)
    full.skip_quiet_tiles = False
    quiet = BatchedBicrystals(dims, q, dt, da, base_height=6.0)
    graphed = BatchedBicrystals(dims, q, dt, da, base_height=6.0)
    graphed.capture(10)
    full.step(60, use_graph=False)
    quiet.step(60, use_graph=False)
    graphed.step(60)
    torch.cuda.synchronize()
    for b in (full, quiet, graphed):
        b.check()
    for i in range(len(dims)):
        ref = full.dense(i)
        assert np.array_equal(quiet.dense(i), ref), f"instance {i}"
        assert np.array_equal(graphed.dense(i), ref), f"instance {i} (graph)"
    assert int(quiet.tile_flags.sum()) > 0  # uniform warp tiles were recorded


def test_graph_replay_equals_eager():
    a, _ = make_batch()
    a.step(8, use_graph=False)
    g, _ = make_batch()
    g.capture(4)
    g.step(8)
    torch.cuda.synchronize()
    for i in range(len(DIMS)):
        assert np.array_equal(a.dense(i), g.dense(i))


def test_observables_match_host_reductions():
    b, _ = make_batch()
    b.step(10, use_graph=False)
    hl, hr, v1, v2 = b.fronts()
    for i, (nx, ny, nz) in enumerate(DIMS):
        phi = b.dense(i).astype(np.float64)
        solid = 1.0 - phi[0]
        mask = solid > 0.5
        has = mask.any(axis=2)
        top = np.where(has, nz - 1 - np.argmax(mask[:, :, ::-1], axis=2), -1)
        split = nx // 2
        left = top[:split][has[:split]]
        right = top[split:][has[split:]]
        assert math.isclose(hl[i], left.mean(), rel_tol=0, abs_tol=1e-9)
        assert math.isclose(hr[i], right.mean(), rel_tol=0, abs_tol=1e-9)
        assert math.isclose(v1[i], phi[1].sum(), rel_tol=1e-6)
        assert math.isclose(v2[i], phi[2].sum(), rel_tol=1e-6)
    ang = b.gb_inclination(z_from=0)
    assert np.all(np.isfinite(ang)) and np.all(np.abs(ang) < 45.0)


def test_every_work_list_shape_gives_the_same_batch(tmp_path, monkeypatch):
    """The batched step's work-list kernel shapes (the autotuner's candidates)
    only reschedule the work: results bit identical; the tuner restores the
    state it timed on and caches its pick."""
    from mpf3d import autotune
    monkeypatch.setenv("MPF3D_TUNING_CACHE", str(tmp_path / "tuning.json"))
    ref, _ = make_batch()
    ref.step(6, use_graph=False)
    for cfg in [(4, 8, 4, 256, 4, 128), (4, 8, 32, 128, 32, 64), (4, 8, 16, 128, 16, 64)]:
        b, _ = make_batch()
        b.tuning = autotune.make(cfg)
        b.step(6, use_graph=False)
        for i in range(len(DIMS)):
            assert np.array_equal(b.dense(i), ref.dense(i)), cfg
    b, _ = make_batch()
    before = [b.dense(i) for i in range(len(DIMS))]
    rec = b.autotune(steps=2)
    assert all(np.array_equal(b.dense(i), before[i]) for i in range(len(DIMS)))
    assert rec["ms_per_step"] <= rec["default_ms_per_step"]
    b.step(6, use_graph=False)
    for i in range(len(DIMS)):
        assert np.array_equal(b.dense(i), ref.dense(i))
    assert (tmp_path / "tuning.json").exists()
