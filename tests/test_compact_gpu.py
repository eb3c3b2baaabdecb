"""Compact FP32 fused stepper against the FP64 oracle (reference numerics
with float64 phi and scalars).  Tolerance: max|dphi| <= 1e-4, the FP32 bar
of the hot path; active-phase lists of the initial state exact."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

TOL = 1e-4


def oracle_fp64(case, steps, aniso=True, torque=True):
    phi0 = case.phi.astype(np.float64)
    temp0 = case.temp.astype(np.float64)
    sc = O.make_scalars([float(v) for v in case.phys.kernel_scalars(f32=False)], False)
    rate = case.phys.derived()["cooling_rate"]
    phi, _, nf, _ = O.run(phi0, temp0, case.wij, case.aij, case.mij, case.n111, sc, steps,
                          cooling_rate=rate, rate_f32=False, switchable=True, aniso=int(aniso),
                          torque=int(torque))
    return phi, nf


def make_solver(case, **kw):
    from mpf3d.solver import CompactSolver
    return CompactSolver(case.phi, case.temp, case.n111, case.wij, case.aij, case.mij, case.phys, **kw)


def test_dense_compact_round_trip_is_exact():
    from mpf3d import inputs
    case = inputs.voronoi_case(20, 12, 18, 6, 6, seed=2)
    s = make_solver(case)
    back = s.to_dense()
    assert np.array_equal(back, case.phi)
    nf = s.active_count()
    mf = np.zeros((50,) + case.phi.shape[1:], np.int32)
    onf = np.zeros(case.phi.shape[1:], np.int32)
    O.apt(case.phi, mf, onf, np.zeros(2, np.int32))
    assert np.array_equal(nf, onf)


@pytest.mark.parametrize("aniso,torque", [(True, True), (True, False), (False, False)])
def test_fp32_step_matches_fp64_oracle(aniso, torque):
    from mpf3d import inputs
    case = inputs.voronoi_case(24, 16, 24, 6, 8, seed=4, orientation_seed=9)
    steps = 5
    ref, ref_nf = oracle_fp64(case, steps, aniso, torque)
    s = make_solver(case, anisotropy=aniso, torque=torque)
    s.step(steps)
    got = s.to_dense(np.float64)
    err = np.abs(got - ref).max()
    assert err <= TOL, f"max|dphi| = {err:.3e}"
    assert np.abs(got.sum(axis=0) - 1.0).max() < 1e-5


def test_eight_normal_kernels_equal_four_normal_kernels():
    """For the reference's antipodal {111} sets the interface kernels search 4
    normals; the 8-normal build must give the same state bit for bit (|cos|
    ties exactly within an antipodal pair, the first maximum is kept)."""
    from mpf3d import inputs
    case = inputs.voronoi_case(24, 16, 24, 6, 8, seed=4, orientation_seed=9)
    a, b = make_solver(case), make_solver(case)
    assert a.symmetric_normals
    b.symmetric_normals = False
    a.step(6)
    b.step(6)
    assert np.array_equal(a.to_dense(), b.to_dense())


def test_fp32_step_with_general_normals_matches_fp64_oracle():
    """Normals that are not antipodal pairs (rows 4..7 turned off their
    pairs) run the 8-normal kernels; they still match the FP64 oracle."""
    from mpf3d import inputs
    base = inputs.voronoi_case(24, 16, 24, 6, 8, seed=4, orientation_seed=9)
    rng = np.random.default_rng(3)
    n111 = base.n111.astype(np.float64).copy()
    n111[:, 4:8] += rng.normal(scale=0.2, size=n111[:, 4:8].shape)
    n111 /= np.linalg.norm(n111, axis=2, keepdims=True)
    case = inputs.Case(base.phi, base.temp, base.quats, n111.astype(np.float32), base.wij, base.aij, base.mij,
                       base.phys)
    steps = 5
    ref, _ = oracle_fp64(case, steps)
    s = make_solver(case)
    assert not s.symmetric_normals
    s.step(steps)
    err = np.abs(s.to_dense(np.float64) - ref).max()
    assert err <= TOL, f"max|dphi| = {err:.3e}"


def test_fp32_undercooled_junctions():
    from mpf3d import inputs
    case = inputs.voronoi_case(20, 20, 20, 10, 8, seed=7, orientation_seed=3, undercooling=3.0)
    steps = 4
    ref, _ = oracle_fp64(case, steps)
    s = make_solver(case)
    s.step(steps)
    err = np.abs(s.to_dense(np.float64) - ref).max()
    assert err <= TOL, f"max|dphi| = {err:.3e}"


def test_slot_overflow_is_reported():
    from mpf3d import inputs
    from mpf3d.solver import SlotOverflow
    phi = np.zeros((7, 6, 6, 6), np.float32)
    phi[1:, 2, 2, 2] = 1.0 / 6.0
    phi[0] = np.clip(1.0 - phi[1:].sum(axis=0), 0.0, 1.0)
    case = inputs.voronoi_case(6, 6, 6, 6, 3, seed=1)
    with pytest.raises(SlotOverflow):
        make_solver(inputs.Case(phi, case.temp, case.quats, case.n111, case.wij, case.aij, case.mij),
                    slots=4)


def test_slot_template_widens_instead_of_dropping_phases():
    """Start with 4 slots on a junction-rich case: the solver must widen its
    template and give the same result as a run that started with 16."""
    from mpf3d import inputs
    case = inputs.voronoi_case(20, 20, 16, 12, 6, seed=5, orientation_seed=2, undercooling=2.0)
    a = make_solver(case, slots=4)
    a.step(6, check_every=3)
    b = make_solver(case, slots=16)
    b.step(6)
    assert np.array_equal(a.to_dense(), b.to_dense())
    # the same with the steps replayed from a captured graph: the overflow
    # rolls back to eager steps on the widened buffers
    c = make_solver(case, slots=4)
    c.capture(2)
    c.step(6, check_every=2)
    assert c.slots > 4 and c.graph is None
    assert np.array_equal(c.to_dense(), b.to_dense())


def test_owner_map_start_equals_dense_start():
    """The owner-map initializer builds the same state as converting the
    dense field of the same owner map and profile."""
    from mpf3d import inputs
    from mpf3d.solver import CompactSolver
    phys = inputs.Physics()
    d = phys.derived()
    nx, ny, nz, n, slab = 24, 20, 30, 7, 8
    owner = inputs.voronoi_slab_owner(nx, ny, nz, n, slab, seed=9)
    prof = inputs.tanh_profile(nz, slab, phys.dx, d["delta"])
    phi = inputs.phi_from_owner(owner, n, prof)
    temp = inputs.temperature_field(nx, ny, nz, phys.T_melt, phys.G, phys.dx, slab)
    q = inputs.random_quaternions(n, 4)
    wij, aij, mij = inputs.matrices_for(phys, n + 1)
    n111 = inputs.rotated_n111(q)
    a = CompactSolver(phi, temp, n111, wij, aij, mij, phys)
    b = CompactSolver.from_owner(owner[:, :, :slab], prof, temp, n111, wij, aij, mij, phys)
    assert np.array_equal(a.to_dense(), b.to_dense())
    a.step(3)
    b.step(3)
    assert np.array_equal(a.to_dense(), b.to_dense())


def test_every_launch_shape_gives_the_same_state(tmp_path, monkeypatch):
    """The autotuner's candidates only reschedule the work: results are bit
    identical; the tuner restores the state it timed on and caches its pick."""
    from mpf3d import autotune, inputs
    monkeypatch.setenv("MPF3D_TUNING_CACHE", str(tmp_path / "tuning.json"))
    case = inputs.voronoi_case(40, 24, 36, 7, 10, seed=12, orientation_seed=1)
    ref = make_solver(case)
    ref.step(4)
    want = ref.to_dense()
    for cfg in [(2, 4, 4, 256, 4, 128), (8, 16, 32, 128, 32, 64), (4, 8, 16, 128, 16, 64)]:
        s = make_solver(case)
        s.tuning = autotune.make(cfg)
        s.step(4)
        assert np.array_equal(s.to_dense(), want), cfg
    s = make_solver(case)
    before = s.to_dense()
    rec = s.autotune(steps=2)
    assert np.array_equal(s.to_dense(), before)
    assert len(rec["config"]) == 6 and rec["ms_per_step"] <= rec["default_ms_per_step"]
    s.step(4)
    assert np.array_equal(s.to_dense(), want)
    assert (tmp_path / "tuning.json").exists()


@pytest.mark.parametrize("cfg", [None, (2, 16, 32, 128, 32, 64), (8, 4, 8, 256, 8, 128)])
def test_quiet_tile_skipping_changes_nothing(cfg):
    """Skipping tiles that stayed uniform (with their neighbours) gives the
    same state, bit for bit, as visiting every cell: over a moving front,
    across a launch-shape change in the middle of the run and after a
    restore from a snapshot."""
    from mpf3d import autotune, inputs
    case = inputs.voronoi_case(72, 20, 64, 6, 10, seed=21, orientation_seed=3, undercooling=1.5)
    a = make_solver(case)
    b = make_solver(case)
    b.skip_quiet_tiles = False
    if cfg is not None:
        a.tuning = autotune.make(cfg)
        b.tuning = autotune.make(cfg)
    quiet_seen = 0.0
    for chunk in range(6):
        a.step(10)
        b.step(10)
        assert np.array_equal(a.to_dense(), b.to_dense()), f"after {10 * (chunk + 1)} steps"
        n = int(a.tile_flags.numel())
        quiet_seen = max(quiet_seen, float(a.tile_flags.float().sum().item()) / n)
        if chunk == 2:  # a shape change in the middle resets the tile history
            a.tuning = autotune.make((4, 8, 8, 256, 8, 128) if cfg is None else (2, 8, 16, 128, 16, 64))
    assert quiet_seen > 0.2  # most of the liquid is skipped
    snap = [t.clone() for t in a.buf[a.cur]]
    a.step(5)
    for dst, src in zip(a.buf[a.cur], snap):  # writing the state from outside ...
        dst.copy_(src)
    a.forget_history()  # ... requires forgetting the step history
    a.step_count -= 5
    b.step(5)
    a.step(5)
    assert np.array_equal(a.to_dense(), b.to_dense())


def test_two_stream_step_replays_from_a_cuda_graph():
    """The step runs its interface kernel on the library's second stream;
    after mpf3d_streams_prepare, two steps captured into a CUDA graph (the
    fork/join is captured with them) and replayed give the eager state bit
    for bit."""
    from mpf3d import _lib, inputs
    case = inputs.voronoi_case(32, 24, 32, 8, 10, seed=5, orientation_seed=2, undercooling=2.0)
    a, b = make_solver(case), make_solver(case)
    a.step(2, check=False)
    dev = torch.device("cuda:0")
    s = torch.cuda.Stream(dev)
    s.wait_stream(torch.cuda.current_stream(dev))
    _lib.check(_lib.lib().mpf3d_streams_prepare(s.cuda_stream), "streams_prepare")
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        b.launch_step(1)
        b.launch_step(2)
    torch.cuda.current_stream(dev).wait_stream(s)
    g.replay()
    torch.cuda.synchronize()
    b.step_count = 2
    assert np.array_equal(a.to_dense(), b.to_dense())
    a.check()
    b.check()


def test_solvers_on_independent_streams():
    """Two solvers stepped on two streams (each with its own second stream
    for the interface kernel), interleaved from the host, give the state of
    a solver stepped alone, bit for bit."""
    from mpf3d import inputs
    case = inputs.voronoi_case(32, 24, 32, 8, 10, seed=5, orientation_seed=2, undercooling=2.0)
    ref, a, b = make_solver(case), make_solver(case), make_solver(case)
    ref.step(6, check=False)
    dev = torch.device("cuda:0")
    s1, s2 = torch.cuda.Stream(dev), torch.cuda.Stream(dev)
    s1.wait_stream(torch.cuda.current_stream(dev))
    s2.wait_stream(torch.cuda.current_stream(dev))
    for _ in range(6):
        with torch.cuda.stream(s1):
            a.step(1, check=False)
        with torch.cuda.stream(s2):
            b.step(1, check=False)
    torch.cuda.synchronize()
    want = ref.to_dense()
    assert np.array_equal(a.to_dense(), want)
    assert np.array_equal(b.to_dense(), want)
    for s in (ref, a, b):
        s.check()


def test_device_clock_equals_temperature_by_value():
    """mpf3d_compact_step_clocked (temperature from the device step clock)
    gives the state of mpf3d_compact_step_tuned with T_melt + s * rate passed
    by value, bit for bit, under fast cooling."""
    import ctypes
    from mpf3d import _lib, inputs
    case = inputs.voronoi_case(32, 24, 32, 8, 10, seed=5, orientation_seed=2, undercooling=1.0)
    a, b = make_solver(case, cooling_rate=0.37), make_solver(case, cooling_rate=0.37)
    a.step(7, check=False)  # the solver's own stepping: the clocked entry
    for s in range(1, 8):
        src, dst = b.buf[b.cur], b.buf[1 - b.cur]
        rc = _lib.lib().mpf3d_compact_step_tuned(
            src[0].data_ptr(), src[1].data_ptr(), src[2].data_ptr(), dst[0].data_ptr(), dst[1].data_ptr(),
            dst[2].data_ptr(), b.slots, b.amax, b.T0z.data_ptr(), b.T_melt + s * b.cooling_rate,
            b.wij.data_ptr(), b.a2ij.data_ptr(), b.mij.data_ptr(), b.n111.data_ptr(), b.N, b.nx, b.ny, b.nz,
            ctypes.byref(b.scalars), 1, 1, int(b.symmetric_normals), b.work_items.data_ptr(),
            b.work_count.data_ptr(), s & 1, b.err.data_ptr(), b._stream(), None, b.tile_flags.data_ptr(),
            _lib.STEP_MULTI_LIST)
        _lib.check(rc, "compact_step_tuned")
        b.cur = 1 - b.cur
    assert np.array_equal(a.to_dense(), b.to_dense())
    a.check()
    b.check()


def test_captured_steps_replay_repeatedly_and_keep_cooling():
    """capture(4) then step(13): three graph replays and one eager step, with
    eager steps before; the temperature keeps falling across replays (the
    device clock), so the state equals 14 eager steps bit for bit.  With fast
    cooling a replay that repeated the captured temperatures would differ."""
    from mpf3d import inputs
    case = inputs.voronoi_case(32, 24, 32, 8, 10, seed=5, orientation_seed=2, undercooling=1.0)
    a, b = make_solver(case, cooling_rate=0.37), make_solver(case, cooling_rate=0.37)
    a.sweep_tma = b.sweep_tma = True
    a.step(14, check=False)
    b.step(1, check=False)
    b.capture(4)
    b.step(13)
    torch.cuda.synchronize()
    assert b.step_count == 14
    assert np.array_equal(a.to_dense(), b.to_dense())
    a.check()
    b.check()


def test_pinned_host_conversion_in_place():
    """Dense phi in pinned host memory is converted in place over the CPU-GPU
    link (no device copy) and written back in place: the state and the
    written field equal those of the device-memory path."""
    from mpf3d import inputs
    case = inputs.voronoi_case(40, 24, 36, 7, 10, seed=12, orientation_seed=1)
    pinned = torch.from_numpy(case.phi).pin_memory()
    a = make_solver(case)
    from mpf3d.solver import CompactSolver
    b = CompactSolver(pinned, case.temp, case.n111, case.wij, case.aij, case.mij, case.phys)
    assert np.array_equal(a.to_dense(), b.to_dense())
    a.step(3)
    b.step(3)
    out = torch.empty(case.phi.shape, dtype=torch.float32).pin_memory()
    out.fill_(-1.0)
    r = b.to_dense(out=out)
    torch.cuda.synchronize()
    assert r is out
    assert np.array_equal(out.numpy(), a.to_dense())
    with pytest.raises(ValueError):
        b.to_dense(out=torch.empty(case.phi.shape, dtype=torch.float32))  # not pinned


@pytest.mark.parametrize("shape,cfg", [((72, 20, 64), None), ((36, 13, 30), (8, 4, 8, 256, 8, 128)),
                                       ((64, 24, 40), (2, 16, 32, 128, 32, 64))])
def test_tma_staged_sweep_changes_nothing(shape, cfg):
    """The sweep with each block's heads staged in shared memory by one TMA
    copy (periodic x/y halos patched in, clamped z) classifies exactly like
    the plain sweep: the states agree bit for bit over a moving front with
    quiet tiles, on domains whose x and y extents are not multiples of the
    block (partial edge tiles)."""
    from mpf3d import autotune, inputs
    nx, ny, nz = shape
    case = inputs.voronoi_case(nx, ny, nz, 6, 10, seed=21, orientation_seed=3, undercooling=1.5)
    a = make_solver(case)
    b = make_solver(case)
    b.sweep_tma = True
    if cfg is not None:
        a.tuning = autotune.make(cfg)
        b.tuning = autotune.make(cfg)
    for chunk in range(4):
        a.step(8)
        b.step(8)
        assert np.array_equal(a.to_dense(), b.to_dense()), f"after {8 * (chunk + 1)} steps"
    b.check()
