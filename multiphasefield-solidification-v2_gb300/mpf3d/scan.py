"""Orientation scan on the batched engine: single-grain spheres growing in an
undercooled melt, one batch instance per orientation case.

The reference (run_orientation_scan_3d.py:495-841) runs one case after
another through the dense kernels and measures on the host every
`save_every` steps.  Here every case is one instance of
``BatchedBicrystals(layout="sphere")``: all cases step together (CUDA-graph
replay between samples) and the observables of measure_observables
(:354-394) -- grain volume, equivalent radius and the directional radii
along x, y, z and [111] -- are reduced on the GPU.  The growth-rate fit and
the anisotropy index (:397-444) run on the host over the short time series,
as in the reference.  Any number of cases fits in one batch, so a scan over
thousands of random orientations is one call.
"""

from __future__ import annotations

import csv
import math
import re

import numpy as np

from .batched import BatchedBicrystals
from .inputs import Physics

DIRECTIONS = {"x": (1.0, 0.0, 0.0), "y": (0.0, 1.0, 0.0), "z": (0.0, 0.0, 1.0), "diag111": (1.0, 1.0, 1.0)}
TIMESERIES_FIELDS = ["step", "time", "volume", "equivalent_radius", "radius_x", "radius_y", "radius_z",
                     "radius_diag111"]
SUMMARY_FIELDS = ["case_name", "orientation_label", "orientation_type", "euler_x_deg", "euler_y_deg",
                  "euler_z_deg", "quat_x", "quat_y", "quat_z", "quat_w", "final_volume", "final_equivalent_radius",
                  "fitted_growth_rate", "anisotropy_index", "fit_start_step", "fit_end_step", "fit_start_time",
                  "fit_end_time", "fit_points"]


def _rotation():
    from scipy.spatial.transform import Rotation

    return Rotation


def align_direction_to_z_quaternion(direction) -> list:
    """Quaternion (x, y, z, w) of the rotation taking `direction` onto +z
    (run_orientation_scan_3d.py:117-122)."""
    R = _rotation()
    src = np.array([direction], np.float64)
    src /= np.linalg.norm(src, axis=1, keepdims=True)
    rot, _ = R.align_vectors(np.array([[0.0, 0.0, 1.0]]), src)
    return rot.as_quat().astype(np.float64).tolist()


def default_orientation_cases() -> list:
    """The reference's five default cases ({100}, {110}, {111}, two mixed;
    run_orientation_scan_3d.py:125-152) as config dicts."""
    return [
        {"label": "{100}", "orientation_type": "euler", "euler_deg": [0.0, 0.0, 0.0]},
        {"label": "{110}", "orientation_type": "euler", "euler_deg": [0.0, 45.0, 0.0]},
        {"label": "{111}", "orientation_type": "quaternion", "quaternion": align_direction_to_z_quaternion([1, 1, 1])},
        {"label": "mid1", "orientation_type": "euler", "euler_deg": [0.0, 15.0, 0.0]},
        {"label": "mid2", "orientation_type": "euler", "euler_deg": [20.0, 35.0, 10.0]},
    ]


def resolve_orientation_cases(raw_cases=None) -> list:
    """Config dicts -> cases with a unit quaternion and its xyz Euler angles
    (run_orientation_scan_3d.py:155-183; orientation_utils.build_quaternion_from_config)."""
    R = _rotation()
    out = []
    for i, raw in enumerate(raw_cases or default_orientation_cases(), start=1):
        if not isinstance(raw, dict):
            raise ValueError(f"orientation_cases[{i - 1}] must be a dict.")
        otype = raw.get("orientation_type", "euler")
        if otype == "euler":
            q = R.from_euler("xyz", raw.get("euler_deg", [0.0, 0.0, 0.0]), degrees=True).as_quat()
        elif otype == "quaternion":
            q = np.asarray(raw["quaternion"], np.float64)
            nrm = np.linalg.norm(q)
            if nrm == 0.0:
                raise ValueError("zero quaternion")
            q = q / nrm
        else:
            raise ValueError(f"unsupported orientation_type {otype!r}")
        import warnings

        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            e = R.from_quat(q).as_euler("xyz", degrees=True)
        out.append({"case_index": i, "label": str(raw.get("label", f"case_{i:02d}")), "orientation_type": otype,
                    "quaternion": [float(v) for v in q], "euler_deg": [float(v) for v in e]})
    return out


def resolve_anisotropy_mode(mode: str, delta_a: float, ksi: float):
    """(enable_anisotropy, enable_torque, delta_a, ksi) of an anisotropy mode
    (run_orientation_scan_3d.py:186-196)."""
    mode = mode.lower()
    if mode == "full":
        return 1, 1, float(delta_a), float(ksi)
    if mode == "isotropic":
        return 0, 0, 0.0, 1.0
    if mode == "energetic_only":
        return 1, 1, float(delta_a), 1.0
    if mode == "kinetic_only":
        return 1, 0, 0.0, float(ksi)
    raise ValueError(f"Unknown aniso_mode: {mode}")


def fit_growth_rate(timeseries, fit_fraction: float, fit_end_time_s=None):
    """Slope of the equivalent radius over time (m/s) over the trailing
    `fit_fraction` of the samples, or over t <= fit_end_time_s when that
    leaves two samples (run_orientation_scan_3d.py:397-432).
    Returns (rate, first index, last index, points)."""
    if len(timeseries) < 2:
        return float("nan"), 0, 0, 0
    times = np.array([float(r["time"]) for r in timeseries], np.float64)
    req = np.array([float(r["equivalent_radius"]) for r in timeseries], np.float64)
    idx = np.arange(len(timeseries))
    ok = np.isfinite(times) & np.isfinite(req)
    if fit_end_time_s is not None and fit_end_time_s > 0.0:
        cut = ok & (times <= fit_end_time_s + 1.0e-15)
        if np.count_nonzero(cut) >= 2:
            sel = idx[cut]
            return float(np.polyfit(times[cut], req[cut], 1)[0]), int(sel[0]), int(sel[-1]), int(cut.sum())
    vi, vt, vr = idx[ok], times[ok], req[ok]
    if vt.size < 2:
        return float("nan"), 0, 0, 0
    n_use = max(2, int(math.ceil(vt.size * fit_fraction)))
    return float(np.polyfit(vt[-n_use:], vr[-n_use:], 1)[0]), int(vi[-n_use]), int(vi[-1]), int(n_use)


def anisotropy_index(row) -> float:
    """(max - min) / mean of the finite directional radii
    (run_orientation_scan_3d.py:435-444)."""
    vals = np.array([float(row.get(k, float("nan"))) for k in ("radius_x", "radius_y", "radius_z",
                                                                  "radius_diag111")])
    vals = vals[np.isfinite(vals)]
    if vals.size < 2:
        return float("nan")
    m = float(np.mean(vals))
    if abs(m) < 1.0e-30:
        return float("nan")
    return float((np.max(vals) - np.min(vals)) / m)


def safe_case_name(label: str) -> str:
    name = re.sub(r"[^A-Za-z0-9._-]+", "_", label.strip())
    return name.strip("_") or "case"


def write_csv(path: str, rows, fields) -> None:
    with open(path, "w", encoding="utf-8", newline="") as f:
        w = csv.DictWriter(f, fieldnames=fields)
        w.writeheader()
        for r in rows:
            w.writerow({k: r.get(k, "") for k in fields})


def run_orientation_scan(cases=None, dims=(96, 96, 96), nsteps: int = 150, save_every: int = 10,
                         radius_cells: float = 10.0, undercooling: float = 1.0, aniso_mode: str = "full",
                         fit_fraction: float = 0.5, fit_end_time_s=None, probe_step_cells: float = 0.5,
                         center_frac=(0.5, 0.5, 0.5), phys: Physics | None = None, slots: int = 4,
                         graph: bool = True, device="cuda:0") -> dict:
    """Grow one sphere per orientation case for `nsteps` steps and fit each
    case's growth rate (the reference's orientation scan, defaults as its
    config: 96^3, 150 steps, samples every 10, radius 10 cells, 1 K,
    aniso_mode "full").  Returns {"cases", "timeseries": {label: rows},
    "summary": rows, "batch"}."""
    if save_every <= 0 or nsteps <= 0:
        raise ValueError("nsteps and save_every must be positive")
    phys = phys or Physics()
    fit_fraction = min(1.0, max(0.1, float(fit_fraction)))
    probe_step_cells = max(0.1, float(probe_step_cells))
    cs = resolve_orientation_cases(cases)
    n = len(cs)
    ea, et, da, ksi = resolve_anisotropy_mode(aniso_mode, phys.delta_a, phys.ksi)
    run_phys = phys.replace(ksi=ksi, delta_a=da)
    quats = np.zeros((n, 2, 4))
    quats[:, 1] = (0.0, 0.0, 0.0, 1.0)
    quats[:, 0] = [c["quaternion"] for c in cs]
    nx, ny, nz = (int(v) for v in dims)
    center = [center_frac[0] * nx, center_frac[1] * ny, center_frac[2] * nz]
    b = BatchedBicrystals([(nx, ny, nz)] * n, quats, np.full(n, undercooling), np.full(n, da), run_phys,
                          slots=slots, anisotropy=bool(ea), torque=bool(et), device=device, layout="sphere",
                          radius=radius_cells, center=center)
    dx, dt = float(phys.dx), float(phys.dt)
    dirs = np.array(list(DIRECTIONS.values()))
    series = [[] for _ in range(n)]

    def sample(step):
        _, _, v1, _ = b.fronts()
        r = b.ray_radii(dirs, threshold=0.5, step_cells=probe_step_cells)
        for i in range(n):
            vol = float(v1[i] * dx ** 3)
            row = {"step": int(step), "time": float(step * dt), "volume": vol,
                   "equivalent_radius": float((3.0 * vol / (4.0 * math.pi)) ** (1.0 / 3.0)) if vol > 0.0 else 0.0}
            for j, name in enumerate(DIRECTIONS):
                row[f"radius_{name}"] = float(r[i, j] * dx) if np.isfinite(r[i, j]) else float("nan")
            series[i].append(row)

    if graph and save_every % 2 == 0:
        b.capture(save_every)
    sample(0)
    done = 0
    while done < nsteps:
        k = min(save_every, nsteps - done)
        b.step(k, use_graph=graph)
        done += k
        sample(done)
    b.check()
    summary = []
    for i, c in enumerate(cs):
        ts = series[i]
        rate, f0, f1, fp = fit_growth_rate(ts, fit_fraction, fit_end_time_s)
        fin = ts[-1]
        e, q = c["euler_deg"], c["quaternion"]
        summary.append({
            "case_name": f"{int(c['case_index']):02d}_{safe_case_name(c['label'])}",
            "orientation_label": c["label"], "orientation_type": c["orientation_type"],
            "euler_x_deg": e[0], "euler_y_deg": e[1], "euler_z_deg": e[2],
            "quat_x": q[0], "quat_y": q[1], "quat_z": q[2], "quat_w": q[3],
            "final_volume": fin["volume"], "final_equivalent_radius": fin["equivalent_radius"],
            "fitted_growth_rate": rate, "anisotropy_index": anisotropy_index(fin),
            "fit_start_step": int(ts[f0]["step"] if fp > 0 else 0), "fit_end_step": int(ts[f1]["step"] if fp > 0 else 0),
            "fit_start_time": float(ts[f0]["time"] if fp > 0 else 0.0),
            "fit_end_time": float(ts[f1]["time"] if fp > 0 else 0.0), "fit_points": int(fp)})
    return {"cases": cs, "timeseries": {c["label"]: series[i] for i, c in enumerate(cs)}, "summary": summary,
            "batch": b}
