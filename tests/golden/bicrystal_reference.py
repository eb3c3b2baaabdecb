"""Loads the interface, groove and bicrystal analysis functions of the
reference's verification suite (tests/verification_3d.py) without its GPU,
plotting and YAML imports: the function definitions are taken from the
source with ``ast`` and executed in a namespace holding numpy, math and
scipy's Rotation.  Test infrastructure only; used by make_golden.py and
make_groove_golden.py at fixture-generation time.
"""
from __future__ import annotations

import ast
import importlib
import math
import os
import sys

import numpy as np

NAMES = [
    "interface_positions_3d", "interface_profile_xz", "groove_angle_from_profile",
    "interface_curve_from_field_xz", "solid_interface_curve_xz", "sample_column_at_fractional_z",
    "boundary_delta_profile_x", "interpolate_root_from_sign_change",
    "grain_boundary_root_and_trijunction", "fit_interface_line", "robust_groove_metrics",
    "compute_metrics_3d", "finalize_metrics", "bicrystal_group_metrics", "bicrystal_phi_3d",
    "alternating_multigrain_phi_3d", "stripe_grain_map", "wavy_single_phi_3d",
    "quaternions_from_rotations", "rotation_align_111_to_z", "orientation_library",
]


def reference_functions(reference_root: str) -> dict:
    path = os.path.join(reference_root, "tests", "verification_3d.py")
    tree = ast.parse(open(path, encoding="utf-8").read(), filename=path)
    keep = [n for n in tree.body if isinstance(n, ast.FunctionDef) and n.name in NAMES]
    missing = set(NAMES) - {n.name for n in keep}
    if missing:
        raise RuntimeError(f"not found in {path}: {sorted(missing)}")
    mod = ast.Module(body=keep, type_ignores=[])
    if reference_root not in sys.path:
        sys.path.insert(0, reference_root)
    from typing import Any, Callable
    from scipy.spatial.transform import Rotation
    s3 = importlib.import_module("src.seed_modes_3d")
    ns = {"np": np, "math": math, "Rotation": Rotation, "Any": Any, "Callable": Callable,
          "init_phi_from_grain_map_3d": s3.init_phi_from_grain_map_3d,
          "__name__": "verification_3d_subset"}
    exec(compile(mod, path, "exec"), ns)
    return {k: ns[k] for k in NAMES}
