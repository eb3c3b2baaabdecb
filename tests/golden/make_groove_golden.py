"""Golden outputs of the reference's interface, groove and bicrystal analysis
(tests/verification_3d.py, loaded by ``bicrystal_reference``) and of its
initial-field builders, written to ``groove_metrics.npz``.

Test infrastructure only.  Usage (needs a checkout of the reference and the
``groove_f32.npz`` golden run made by make_golden.py)::

    python tests/golden/make_groove_golden.py --reference /path/to/multiphasefield-solidification-v2

Contents:
  * the reference's robust_groove_metrics, grain_boundary_root_and_trijunction,
    interface_profile_xz, groove_angle_from_profile, compute_metrics_3d and
    finalize_metrics on every step of the groove_f32 run;
  * the same on synthetic bicrystal and stripe fields (offset, wavy, tilted
    fronts) made by the reference's bicrystal_phi_3d and
    alternating_multigrain_phi_3d, with those fields themselves;
  * bicrystal_group_metrics on a stripe field.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import bicrystal_reference  # noqa: E402

DX = 1.0e-4
DELTA = 6.0 * DX
GROOVE_KEYS = ["root_x_cells", "root_z_cells", "left_angle_deg", "right_angle_deg", "left_fit_rmse",
               "right_fit_rmse", "groove_depth_cells", "dihedral_angle_like_deg"]


def analyse(F, phi0, phi, split, total_time):
    gm = F["robust_groove_metrics"](phi, root_x_guess=float(split))
    root = F["grain_boundary_root_and_trijunction"](phi, 1, 2, x_guess=float(split))
    prof = F["interface_profile_xz"](phi)
    m = F["compute_metrics_3d"](phi, np.zeros(phi.shape[1:], np.int32), DX, 0.0)
    m = F["finalize_metrics"](m, phi0, phi, DX, total_time)
    return {
        "groove": np.array([gm[k] for k in GROOVE_KEYS]),
        "root": np.array([root["root_x_cells"], root["root_z_cells"]]),
        "profile": prof,
        "groove_angle_split": np.array([F["groove_angle_from_profile"](prof, DX, split)]),
        "front": np.array([m["interface_position_mean"], m["interface_position_max"],
                           m["interface_roughness"], m["solid_fraction"], m["solid_volume_growth"],
                           m["front_velocity"], m["winner_loser_volume_ratio"]]),
        "grain_volumes": np.array(m["grain_volumes"]),
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("MPF3D_REFERENCE_ROOT"),
                    required="MPF3D_REFERENCE_ROOT" not in os.environ,
                    help="checkout of the reference (or set MPF3D_REFERENCE_ROOT)")
    args = ap.parse_args()
    F = bicrystal_reference.reference_functions(args.reference)
    out = {"groove_keys": np.array(GROOVE_KEYS)}
    cases = []

    g = np.load(os.path.join(HERE, "groove_f32.npz"))
    phi0 = g["phi0"]
    for s in range(g["phi"].shape[0]):
        cases.append((f"groove_step{s + 1}", phi0, g["phi"][s], 10, 5.0e-5 * (s + 1), None))

    # synthetic bicrystals: grains offset in height, wavy and flat fronts, other splits
    for name, kw in [("offset", dict(left_offset=1.3, right_offset=-0.7, waviness=0.0)),
                     ("wavy", dict(waviness=0.8)),
                     ("wavy_offset", dict(left_offset=-0.9, right_offset=0.4, waviness=1.1))]:
        for split in (7, 12):
            ph = F["bicrystal_phi_3d"](18, 6, 28, DX, DELTA, 7.0, split, **kw)
            base = F["bicrystal_phi_3d"](18, 6, 28, DX, DELTA, 7.0, split)
            cases.append((f"bicrystal_{name}_s{split}", base, ph, split, 4.0e-4, ph))
    # a front tilted across the boundary (linear height), grains 1 | 2 at x = 9
    x = np.arange(20, dtype=np.float64).reshape(20, 1, 1)
    z = np.arange(24, dtype=np.float64).reshape(1, 1, 24)
    h = 6.0 + 0.35 * x - 1.2 * np.exp(-((x - 9.4) ** 2) / 3.0)
    solid = (0.5 * (1.0 - np.tanh(np.float32(2.2 / DELTA) * ((z - h) * DX)))).astype(np.float32)
    tilt = np.zeros((3, 20, 6, 24), np.float32)
    tilt[1, :9] = np.broadcast_to(solid[:9], (9, 6, 24))
    tilt[2, 9:] = np.broadcast_to(solid[9:], (11, 6, 24))
    tilt[0] = np.clip(1.0 - tilt[1] - tilt[2], 0.0, 1.0)
    cases.append(("tilted", F["bicrystal_phi_3d"](20, 6, 24, DX, DELTA, 6.0, 9), tilt, 9, 1.0e-3, tilt))

    names = []
    for name, p0, ph, split, t, field in cases:
        names.append(name)
        for k, v in analyse(F, p0, ph, split, t).items():
            out[f"{name}/{k}"] = v
        if field is not None:
            out[f"{name}/phi"] = field
        out[f"{name}/split"] = np.int32(split)
        out[f"{name}/total_time"] = np.float64(t)
        if field is None:
            out[f"{name}/step"] = np.int32(int(name.split("step")[1]))

    # stripe fields of the multigrain case and their family volumes
    for ng, wav in ((6, 1.5), (6, 0.0), (4, 1.0)):
        key = f"multigrain_{ng}_{str(wav).replace('.', 'p')}"
        ph = F["alternating_multigrain_phi_3d"](24, 10, 30, DX, DELTA, 7.0, ngrains=ng, waviness=wav)
        fam = F["bicrystal_group_metrics"](ph, list(range(1, ng + 1, 2)), list(range(2, ng + 1, 2)), DX)
        out[f"{key}/phi"] = ph
        out[f"{key}/family"] = np.array([fam["volume_a"], fam["volume_b"], fam["winner_loser_volume_ratio"],
                                         1.0 if fam["winner_family"] == "A" else 0.0])
        names.append(key)
    out["stripe_map_18_3"] = F["stripe_grain_map"](18, 4, 3)
    out["stripe_map_24_6"] = F["stripe_grain_map"](24, 10, 6)
    out["quats_library"] = np.stack([r.as_quat() for r in F["orientation_library"]().values()])
    out["library_names"] = np.array(list(F["orientation_library"]().keys()))
    out["cases"] = np.array(names)
    np.savez_compressed(os.path.join(HERE, "groove_metrics.npz"), **out)
    print(json.dumps({"cases": len(names), "bytes": os.path.getsize(os.path.join(HERE, "groove_metrics.npz"))}))


if __name__ == "__main__":
    main()
