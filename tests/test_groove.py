"""Groove, trijunction and bicrystal analysis (mpf3d.groove) and the
verification suite's initial fields (mpf3d.inputs) against the reference's
own functions (tests/golden/groove_metrics.npz, made by
tests/golden/make_groove_golden.py), and the groove_f32 golden run against
the values the reference recorded for groove_depth_only and
robust_groove_angle_estimation (tests/verification_report.md:97-108)."""
import math

import numpy as np
import pytest

from mpf3d import groove, inputs
from _helpers import GOLDEN

DX = 1.0e-4
DELTA = 6.0 * DX


@pytest.fixture(scope="module")
def fx():
    return np.load(f"{GOLDEN}/groove_metrics.npz")


def _close(a, b, rel=1e-9, abs_=1e-12):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    assert a.shape == b.shape
    both_nan = np.isnan(a) & np.isnan(b)
    assert np.array_equal(np.isnan(a), np.isnan(b)), (a, b)
    ok = both_nan | (np.abs(a - b) <= abs_ + rel * np.abs(b))
    assert ok.all(), (a, b)


def _cases(fx):
    return [str(c) for c in fx["cases"] if not str(c).startswith("multigrain")]


def _field(fx, name):
    if f"{name}/phi" in fx.files:
        return fx[f"{name}/phi"]
    g = np.load(f"{GOLDEN}/groove_f32.npz")
    return g["phi"][int(fx[f"{name}/step"]) - 1]


def _initial(fx, name):
    if name.startswith("groove_step"):
        return np.load(f"{GOLDEN}/groove_f32.npz")["phi0"]
    if name == "tilted":
        return inputs.bicrystal_field(20, 6, 24, DX, DELTA, 6.0, 9)
    return inputs.bicrystal_field(18, 6, 28, DX, DELTA, 7.0, int(fx[f"{name}/split"]))


def test_groove_metrics_match_reference(fx):
    keys = [str(k) for k in fx["groove_keys"]]
    for name in _cases(fx):
        phi = _field(fx, name)
        split = int(fx[f"{name}/split"])
        gm = groove.groove_metrics(phi, root_x_guess=float(split))
        # slopes come from a closed-form least-squares fit rather than polyfit
        _close([gm[k] for k in keys], fx[f"{name}/groove"], rel=1e-9, abs_=1e-9)
        r = groove.grain_boundary_root(phi, 1, 2, x_guess=float(split))
        _close([r["root_x_cells"], r["root_z_cells"]], fx[f"{name}/root"])
        prof = groove.interface_profile_xz(phi)
        assert np.array_equal(prof, fx[f"{name}/profile"], equal_nan=True)
        _close([groove.groove_angle_from_profile(prof, DX, split)], fx[f"{name}/groove_angle_split"])


def test_front_summary_matches_reference(fx):
    for name in _cases(fx):
        phi = _field(fx, name)
        s = groove.run_summary(_initial(fx, name), phi, DX, float(fx[f"{name}/total_time"]))
        got = [s["interface_position_mean"], s["interface_position_max"], s["interface_roughness"],
               s["solid_fraction"], s["solid_volume_growth"], s["front_velocity"],
               s["winner_loser_volume_ratio"]]
        _close(got, fx[f"{name}/front"], rel=1e-12, abs_=1e-18)
        _close(s["grain_volumes"], fx[f"{name}/grain_volumes"], rel=1e-12, abs_=0.0)


def test_initial_fields_match_reference_builders(fx):
    for name in _cases(fx):
        if not name.startswith("bicrystal_"):
            continue
        kind, split = name[len("bicrystal_"):].rsplit("_s", 1)
        kw = {"offset": dict(left_offset=1.3, right_offset=-0.7, waviness=0.0),
              "wavy": dict(waviness=0.8),
              "wavy_offset": dict(left_offset=-0.9, right_offset=0.4, waviness=1.1)}[kind]
        got = inputs.bicrystal_field(18, 6, 28, DX, DELTA, 7.0, int(split), **kw)
        assert np.array_equal(got, fx[f"{name}/phi"]), name
    for ng, wav in ((6, 1.5), (6, 0.0), (4, 1.0)):
        key = f"multigrain_{ng}_{str(wav).replace('.', 'p')}"
        ph = inputs.alternating_multigrain_field(24, 10, 30, DX, DELTA, 7.0, ng, wav)
        assert np.array_equal(ph, fx[f"{key}/phi"]), key
        fam = groove.family_volumes(ph, range(1, ng + 1, 2), range(2, ng + 1, 2), DX)
        _close([fam["volume_a"], fam["volume_b"], fam["winner_loser_volume_ratio"],
                1.0 if fam["winner_family"] == "A" else 0.0], fx[f"{key}/family"], rel=1e-12, abs_=0.0)
    assert np.array_equal(inputs.stripe_grain_map(18, 4, 3), fx["stripe_map_18_3"])
    assert np.array_equal(inputs.stripe_grain_map(24, 10, 6), fx["stripe_map_24_6"])


def test_orientation_library_matches_reference(fx):
    pytest.importorskip("scipy")
    lib = inputs.orientation_library()
    assert list(lib) == [str(n) for n in fx["library_names"]]
    _close(np.stack([r.as_quat() for r in lib.values()]), fx["quats_library"], rel=0.0, abs_=1e-12)


def test_groove_run_reproduces_recorded_reference_values():
    """The 20-step groove_f32 golden run (the reference's kernel source) gives
    the groove metrics the reference recorded on its GPU run of
    groove_depth_only: root (9.5, 6.140266745898822) cells, depth
    1.044794920156776 cells, dihedral-like angle 19.20117935659593 deg, and
    the angle history of robust_groove_angle_estimation (every 2 steps)."""
    g = np.load(f"{GOLDEN}/groove_f32.npz")
    phi = g["phi"][-1]
    gm = groove.groove_metrics(phi, root_x_guess=10.0)
    assert gm["root_x_cells"] == 9.5
    assert gm["root_z_cells"] == pytest.approx(6.140266745898822, rel=1e-12)
    assert gm["groove_depth_cells"] == pytest.approx(1.044794920156776, rel=1e-12)
    assert gm["dihedral_angle_like_deg"] == pytest.approx(19.20117935659593, rel=1e-9)
    assert gm["left_angle_deg"] == pytest.approx(-10.57752338207936, rel=1e-9)
    assert gm["right_angle_deg"] == pytest.approx(8.623655974516568, rel=1e-9)
    assert max(gm["left_fit_rmse"], gm["right_fit_rmse"]) == pytest.approx(0.006562300317471668, rel=1e-6)
    hist = [groove.groove_metrics(g["phi"][s - 1], root_x_guess=10.0)["dihedral_angle_like_deg"]
            for s in range(2, 21, 2)]
    want = [14.459181221271223, 14.661731290308964, 15.035149861886143, 15.530506939995853,
            16.110621306914986, 16.736929566158693, 17.379949177165766, 18.017309905623254,
            18.629417911288115, 19.20117935659593]
    assert hist == pytest.approx(want, rel=1e-9)
    s = groove.run_summary(g["phi0"], phi, DX, 20 * 5.0e-5)
    assert s["interface_position_mean"] == pytest.approx(6.450e-04, rel=1e-12)
    assert s["interface_position_max"] == pytest.approx(7.0e-04, rel=1e-12)
    assert s["solid_fraction"] == pytest.approx(0.3070, abs=5e-5)
    assert s["winner_loser_volume_ratio"] == pytest.approx(1.015, abs=5e-4)
    assert s["front_velocity"] == 0.0


def test_fit_line_and_root_edge_cases():
    x = np.arange(6, dtype=np.float64)
    z = 2.0 + 0.5 * x
    f = groove.fit_line(x, z, 1.0, 4.0)
    assert f["slope"] == pytest.approx(0.5) and f["rmse"] == pytest.approx(0.0, abs=1e-12)
    assert f["angle_deg"] == pytest.approx(math.degrees(math.atan(0.5)))
    assert math.isnan(groove.fit_line(x, z, 10.0, 20.0)["slope"])
    z2 = z.copy()
    z2[2:] = np.nan
    assert math.isnan(groove.fit_line(x, z2, 1.0, 4.0)["angle_deg"])
    # exact zero of delta, and no sign change at all
    assert groove.root_from_sign_change(x, z, np.array([1.0, 0.0, -1.0, -2, -3, -4])) == (1.0, 2.5)
    assert all(math.isnan(v) for v in groove.root_from_sign_change(x, z, np.ones(6)))
    # a column with no solid gives nan in the profile and the curve
    phi = inputs.bicrystal_field(8, 2, 10, DX, DELTA, 4.0, 4)
    phi[0, 3] = 1.0
    phi[1:, 3] = 0.0
    assert np.isnan(groove.interface_profile_xz(phi)[3])
    assert np.isnan(groove.solid_interface_curve_xz(phi)[1][3])
