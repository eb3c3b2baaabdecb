"""Grain-boundary groove, trijunction and bicrystal metrics on a dense phase
field phi[N, nx, ny, nz] (host arrays; one x-z slice is all they read).

Restates the analysis of the reference's verification suite,
tests/verification_3d.py:
  interface_profile_xz            :419-429   integer front height per column
  groove_angle_from_profile       :432-441
  interface_curve_from_field_xz   :444-465   linear phi = 0.5 crossing
  solid_interface_curve_xz        :468-472
  sample_column_at_fractional_z   :475-483
  boundary_delta_profile_x        :486-497
  interpolate_root_from_sign_change :500-528
  grain_boundary_root_and_trijunction :531-545
  fit_interface_line              :548-568
  robust_groove_metrics           :571-609
  finalize_metrics                :657-704   (volume growth, front velocity,
                                              winner/loser ratio, root shift)
  bicrystal_group_metrics         :1366-1381
The slice is the middle y plane unless y_index is given; heights are in
cells, counted along z.
"""
from __future__ import annotations

import math

import numpy as np

NAN = float("nan")


def _mid(ny: int, y_index) -> int:
    return ny // 2 if y_index is None else int(np.clip(y_index, 0, ny - 1))


def _last_true(mask: np.ndarray):
    """Per row of a 2D mask: whether any entry is set and the index of the
    last one."""
    n = mask.shape[1]
    has = mask.any(axis=1)
    return has, n - 1 - np.argmax(mask[:, ::-1], axis=1)


def interface_profile_xz(phi: np.ndarray, y_index=None, threshold: float = 0.5) -> np.ndarray:
    """Highest z with solid fraction above the threshold, per x (nan where the
    column holds no solid)."""
    solid = 1.0 - phi[0][:, _mid(phi.shape[2], y_index), :]
    has, k = _last_true(solid > threshold)
    return np.where(has, k, np.nan).astype(np.float64)


def groove_angle_from_profile(profile: np.ndarray, dx: float, center_idx: int) -> float:
    """Mean of the two one-sided slopes' angles at center_idx (degrees), the
    profile difference taken per dx."""
    if center_idx <= 0 or center_idx >= profile.size - 1:
        return NAN
    left = profile[center_idx] - profile[center_idx - 1]
    right = profile[center_idx + 1] - profile[center_idx]
    if not (np.isfinite(left) and np.isfinite(right)):
        return NAN
    scale = max(dx, 1.0e-30)
    return 0.5 * (math.degrees(math.atan(abs(left) / scale)) + math.degrees(math.atan(abs(right) / scale)))


def interface_curve_xz(field_xz: np.ndarray, threshold: float = 0.5):
    """(x, z) of the field's last crossing of the threshold along z, linearly
    interpolated between the last cell at or above it and the next one."""
    nx, nz = field_xz.shape
    has, k0 = _last_true(field_xz >= threshold)
    z = np.full(nx, np.nan)
    k1 = np.minimum(k0 + 1, nz - 1)
    rows = np.arange(nx)
    v0 = field_xz[rows, k0].astype(np.float64)
    v1 = field_xz[rows, k1].astype(np.float64)
    flat = np.abs(v1 - v0) < 1.0e-12
    with np.errstate(divide="ignore", invalid="ignore"):
        frac = np.where(flat, 0.0, (threshold - v0) / np.where(flat, 1.0, v1 - v0))
    z = np.where(k0 >= nz - 1, float(nz - 1), k0 + frac)
    z[~has] = np.nan
    return np.arange(nx, dtype=np.float64), z


def solid_interface_curve_xz(phi: np.ndarray, y_index=None, threshold: float = 0.5):
    solid = 1.0 - phi[0]
    return interface_curve_xz(solid[:, _mid(solid.shape[1], y_index), :], threshold)


def sample_at_height(col: np.ndarray, z: float) -> float:
    """Linear interpolation of a column at fractional height z (clamped).
    The weights are rounded to the column's precision and the sum is formed
    in it, as the reference's numpy-2 scalar arithmetic does (a float32
    field gives float32 samples)."""
    if not np.isfinite(z):
        return NAN
    nz = col.shape[0]
    z0 = int(np.clip(int(np.floor(z)), 0, nz - 1))
    z1 = min(z0 + 1, nz - 1)
    f = float(z - z0)
    t = col.dtype.type
    return float(t(1.0 - f) * col[z0] + t(f) * col[z1])


def boundary_delta_profile_x(phi: np.ndarray, gid_left: int, gid_right: int, y_index=None):
    """Front curve and, on it, phi_left - phi_right per x."""
    x, z = solid_interface_curve_xz(phi, y_index)
    y = _mid(phi.shape[2], y_index)
    diff = phi[gid_left, :, y, :] - phi[gid_right, :, y, :]
    delta = np.array([sample_at_height(diff[i], z[i]) for i in range(phi.shape[1])])
    return x, z, delta


def root_from_sign_change(x: np.ndarray, z: np.ndarray, delta: np.ndarray, x_guess=None):
    """Zero crossings of delta between neighbouring columns (or columns where
    it is exactly 0), with z interpolated the same way; the one nearest
    x_guess (the middle one without a guess)."""
    roots = []
    for i in range(len(x) - 1):
        d0, d1 = delta[i], delta[i + 1]
        if not (np.isfinite(d0) and np.isfinite(d1)):
            continue
        if d0 == 0.0:
            roots.append((float(x[i]), float(z[i])))
            continue
        if d0 * d1 > 0.0:
            continue
        f = abs(d0) / max(abs(d0) + abs(d1), 1.0e-12)
        zr = (1.0 - f) * z[i] + f * z[i + 1] if (np.isfinite(z[i]) and np.isfinite(z[i + 1])) else NAN
        roots.append((float(x[i] + f * (x[i + 1] - x[i])), float(zr)))
    if not roots:
        return NAN, NAN
    if x_guess is None:
        return roots[len(roots) // 2]
    return min(roots, key=lambda r: abs(r[0] - x_guess))


def grain_boundary_root(phi: np.ndarray, gid_left: int = 1, gid_right: int = 2, y_index=None,
                        x_guess=None) -> dict:
    """Where the boundary between two grains meets the solid-liquid front."""
    x, z, delta = boundary_delta_profile_x(phi, gid_left, gid_right, y_index)
    rx, rz = root_from_sign_change(x, z, delta, x_guess)
    return {"root_x_cells": float(rx), "root_z_cells": float(rz),
            "trijunction_x_cells": float(rx), "trijunction_z_cells": float(rz)}


def fit_line(x: np.ndarray, z: np.ndarray, x_min: float, x_max: float) -> dict:
    """Least-squares line z = slope x + intercept over the finite points with
    x in [x_min, x_max]; angle = atan(slope) in degrees."""
    m = np.isfinite(z) & (x >= x_min) & (x <= x_max)
    xs, zs = x[m], z[m]
    if xs.size < 2:
        return {"slope": NAN, "intercept": NAN, "angle_deg": NAN, "rmse": NAN}
    xm, zm = xs.mean(), zs.mean()
    sxx = float(np.sum((xs - xm) ** 2))
    slope = float(np.sum((xs - xm) * (zs - zm)) / sxx) if sxx > 0.0 else NAN
    intercept = float(zm - slope * xm)
    rmse = float(np.sqrt(np.mean((slope * xs + intercept - zs) ** 2)))
    return {"slope": slope, "intercept": intercept, "angle_deg": math.degrees(math.atan(slope)), "rmse": rmse}


def groove_metrics(phi: np.ndarray, root_x_guess: float, y_index=None, fit_half_width: float = 4.0,
                   exclude_half_width: float = 1.0) -> dict:
    """Groove at the boundary between grains 1 and 2: its root (trijunction),
    the front's slope angle on each side (fitted over exclude..fit half
    widths from the root), their difference (the dihedral-like angle) and the
    depth below the far-field front."""
    x, z = solid_interface_curve_xz(phi, y_index)
    root = grain_boundary_root(phi, 1, 2, y_index, x_guess=root_x_guess)
    rx, rz = root["root_x_cells"], root["root_z_cells"]
    if not np.isfinite(rx):
        rx = float(root_x_guess)
        rz = float(z[int(np.clip(round(rx), 0, len(z) - 1))])
    left = fit_line(x, z, rx - fit_half_width, rx - exclude_half_width)
    right = fit_line(x, z, rx + exclude_half_width, rx + fit_half_width)
    far = np.isfinite(z) & ((x <= rx - fit_half_width) | (x >= rx + fit_half_width))
    far_z = float(np.mean(z[far])) if far.any() else NAN
    depth = max(far_z - rz, 0.0) if (np.isfinite(far_z) and np.isfinite(rz)) else NAN
    dihedral = (abs(right["angle_deg"] - left["angle_deg"])
                if (np.isfinite(left["angle_deg"]) and np.isfinite(right["angle_deg"])) else NAN)
    return {"root_x_cells": float(rx), "root_z_cells": float(rz),
            "trijunction_x_cells": float(rx), "trijunction_z_cells": float(rz),
            "left_angle_deg": left["angle_deg"], "right_angle_deg": right["angle_deg"],
            "left_fit_rmse": left["rmse"], "right_fit_rmse": right["rmse"],
            "groove_depth_cells": float(depth), "dihedral_angle_like_deg": float(dihedral)}


def front_positions(phi: np.ndarray, threshold: float = 0.5) -> np.ndarray:
    """Highest z with solid above the threshold per (x, y), nan where none."""
    solid = 1.0 - phi[0]
    mask = solid > threshold
    nz = mask.shape[2]
    has = mask.any(axis=2)
    return np.where(has, nz - 1 - np.argmax(mask[:, :, ::-1], axis=2), np.nan).astype(np.float64)


def front_mean(phi: np.ndarray, dx: float) -> float:
    pos = front_positions(phi)
    fin = pos[np.isfinite(pos)]
    return float(np.mean(fin) * dx) if fin.size else NAN


def grain_volumes(phi: np.ndarray, dx: float) -> np.ndarray:
    return np.array([float(phi[g].sum() * dx ** 3) for g in range(1, phi.shape[0])])


def run_summary(phi0: np.ndarray, phi: np.ndarray, dx: float, total_time: float) -> dict:
    """Front statistics and growth of a run from phi0 to phi."""
    pos = front_positions(phi)
    fin = pos[np.isfinite(pos)]
    mean1 = float(np.mean(fin) * dx) if fin.size else NAN
    mean0 = front_mean(phi0, dx)
    vols = grain_volumes(phi, dx)
    out = {"interface_position_mean": mean1,
           "interface_position_max": float(np.max(fin) * dx) if fin.size else NAN,
           "interface_roughness": float(np.std(fin) * dx) if fin.size else NAN,
           "solid_fraction": float(np.mean(1.0 - phi[0])),
           "solid_volume_growth": float(np.sum((1.0 - phi[0]) - (1.0 - phi0[0])) * dx ** 3),
           "front_velocity": ((mean1 - mean0) / max(total_time, 1.0e-30)
                              if (np.isfinite(mean1) and np.isfinite(mean0)) else NAN),
           "grain_volumes": vols,
           "surviving_grains": int(np.sum(vols > dx ** 3)),
           "winner_loser_volume_ratio": NAN}
    big = vols[vols > 0.5 * dx ** 3]
    if big.size >= 2:
        out["winner_loser_volume_ratio"] = float(big.max() / max(big.min(), 1.0e-30))
    return out


def family_volumes(phi: np.ndarray, family_a, family_b, dx: float) -> dict:
    """Summed volumes of two grain families; the larger one wins."""
    vols = grain_volumes(phi, dx)
    va = float(np.sum([vols[g - 1] for g in family_a]))
    vb = float(np.sum([vols[g - 1] for g in family_b]))
    win_a = va >= vb
    ratio = va / max(vb, 1.0e-30) if win_a else vb / max(va, 1.0e-30)
    return {"volume_a": va, "volume_b": vb, "winner_loser_volume_ratio": float(ratio),
            "winner_family": "A" if win_a else "B"}
