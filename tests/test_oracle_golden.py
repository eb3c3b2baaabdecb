"""The oracle against golden vectors made by running the reference's own
kernel source (tests/golden/make_golden.py): bit-exact phi, nf, mf, status
and temperature on every case."""
import numpy as np
import pytest

import oracle as O
from _helpers import golden_files, golden_id, valid_mf_equal


@pytest.mark.parametrize("path", golden_files("run"), ids=golden_id)
def test_oracle_matches_reference_source(path):
    g = np.load(path)
    sc = O.make_scalars(g["scalars"], bool(g["scalars_f32"]))
    phi, temp, nf, mf, hist = O.run(
        g["phi0"], g["temp0"], g["wij"], g["aij"], g["mij"], g["n111"], sc, int(g["steps"]),
        cooling_rate=float(g["cooling_rate"]), rate_f32=bool(g["scalars_f32"]),
        cooling=bool(g["cooling"]), checked=bool(g["checked"]),
        switchable=str(g["kernel"]) == "switchable", aniso=int(g["aniso"]),
        torque=int(g["torque"]), record=True)
    for s, (p, n, m, st, t) in enumerate(hist):
        assert np.array_equal(p, g["phi"][s]), f"phi differs at step {s}"
        assert np.array_equal(n, g["nf"][s]), f"nf differs at step {s}"
        assert valid_mf_equal(m, g["mf"][s], n), f"mf differs at step {s}"
        assert np.array_equal(t, g["temp"][s]), f"temperature differs at step {s}"
        if bool(g["checked"]):
            assert np.array_equal(st, g["status"][s])


@pytest.mark.parametrize("path", golden_files("apt"), ids=golden_id)
def test_oracle_apt_known_answers(path):
    g = np.load(path)
    phi = g["phi0"]
    N = phi.shape[0]
    mf = np.zeros((max(N, 50),) + phi.shape[1:], np.int32)
    nf = np.zeros(phi.shape[1:], np.int32)
    st = np.zeros(2, np.int32)
    assert O.apt(phi, mf, nf, st, checked=True) == 0
    assert np.array_equal(nf, g["nf"])
    assert np.array_equal(st, g["status"])
    assert valid_mf_equal(mf, g["mf"], nf)


def test_overflow_known_answer():
    """52 phases of equal value in one cell: status == [1, 52] and nf clamps
    to KMAX (reference verification case kmax_overflow_detection)."""
    n = 52
    phi = np.zeros((n, 4, 4, 4), np.float32)
    phi[:, 1, 1, 1] = np.float32(1.0 / n)
    phi[0] = np.clip(1.0 - phi[1:].sum(axis=0), 0.0, 1.0)
    mf = np.zeros((n, 4, 4, 4), np.int32)
    nf = np.zeros((4, 4, 4), np.int32)
    st = np.zeros(2, np.int32)
    O.apt(phi, mf, nf, st, checked=True)
    assert st.tolist() == [1, 52]
    assert nf[1, 1, 1] == 50


def test_boundary_probes():
    """x/y wrap and z clamp of the APT (reference case boundary_conditions)."""
    phi = np.zeros((4, 6, 5, 5), np.float32)
    phi[1, 0, 2, 2] = 1.0
    phi[2, 3, 0, 2] = 1.0
    phi[3, 3, 2, 0] = 1.0
    phi[0] = np.clip(1.0 - phi[1:].sum(axis=0), 0.0, 1.0)
    mf = np.zeros((50, 6, 5, 5), np.int32)
    nf = np.zeros((6, 5, 5), np.int32)
    O.apt(phi, mf, nf, np.zeros(2, np.int32), checked=True)
    has = lambda c, g: g in mf[: nf[c], c[0], c[1], c[2]].tolist()
    assert has((5, 2, 2), 1)
    assert has((3, 4, 2), 2)
    assert has((3, 2, 1), 3)
    assert not has((3, 2, 4), 3)


def test_unchecked_apt_reports_depth_overflow():
    phi = np.zeros((6, 3, 3, 3), np.float32)
    phi[:, 1, 1, 1] = 1.0 / 6
    mf = np.zeros((4, 3, 3, 3), np.int32)
    nf = np.zeros((3, 3, 3), np.int32)
    assert O.apt(phi, mf, nf, None, checked=False) == -1


def _run2d_history(g):
    f32 = bool(g["scalars_f32"])
    sc = O.make_scalars(g["scalars"], f32)
    phi, temp = g["phi0"].copy(), g["temp0"].copy()
    N, nx, ny = phi.shape
    mf = np.zeros((20, nx, ny), np.int32)
    nf = np.zeros((nx, ny), np.int32)
    phi_new = phi.copy()
    for s in range(int(g["steps"])):
        if float(g["cooling_rate"]) != 0.0:
            O.temp_step(temp, float(g["cooling_rate"]), f32)
        assert O.apt2d(phi, mf, nf) == 0
        assert O.update2d(phi, phi_new, temp, mf, nf, g["wij"], g["aij"], g["mij"], g["n111"], sc) == 0
        phi, phi_new = phi_new, phi
        yield s, phi, nf, mf, temp


@pytest.mark.parametrize("path", golden_files("run2d"), ids=golden_id)
def test_oracle_2d_matches_reference_source(path):
    """2D kernels (src/gpu_kernels.py): bit-exact phi, nf, mf and temperature
    against the reference's own 2D source on every step."""
    g = np.load(path)
    for s, phi, nf, mf, temp in _run2d_history(g):
        assert np.array_equal(phi, g["phi"][s]), f"phi differs at step {s}"
        assert np.array_equal(nf, g["nf"][s]), f"nf differs at step {s}"
        assert valid_mf_equal(mf, g["mf"][s], nf), f"mf differs at step {s}"
        assert np.array_equal(temp, g["temp"][s]), f"temperature differs at step {s}"


def test_oracle_2d_apt_wraps_x_and_clamps_y():
    """2D APT boundaries: x periodic (a phase at x=0 activates x=nx-1), y
    mirror (a phase at y=0 does not activate y=ny-1)."""
    phi = np.zeros((3, 5, 4), np.float32)
    phi[1, 0, 2] = 1.0
    phi[2, 2, 0] = 1.0
    phi[0] = 1.0 - phi[1:].sum(axis=0)
    mf = np.zeros((20, 5, 4), np.int32)
    nf = np.zeros((5, 4), np.int32)
    assert O.apt2d(phi, mf, nf) == 0
    active = lambda g, l, m: g in mf[: nf[l, m], l, m]
    assert active(1, 4, 2) and active(1, 1, 2) and not active(1, 3, 2)
    assert active(2, 2, 1) and not active(2, 2, 3)
    assert O.apt2d(phi, np.zeros((1, 5, 4), np.int32), nf) == -1
