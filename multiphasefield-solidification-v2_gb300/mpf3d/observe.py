"""Observables, slices and checkpoints of a compact state, computed on the GPU.

* ``metrics`` / ``interface_positions``: compute_metrics_3d and
  interface_positions_3d of the reference (tests/verification_3d.py:409-416,
  612-654), reduced in HBM by ``mpf3d_compact_metrics``; only the reduced
  numbers and one float per column come back to the host.
* ``phase_slice`` / ``save_phase_map_png``: the argmax phase map of
  save_phase_map_slice_3d (src/plot_utils_3d.py:36-72) and the solid
  fraction of save_solid_slice (run_orientation_scan_3d.py:199-223), cut on
  the GPU and written as a PNG without a plotting stack (one pixel per cell,
  the tab20 colour table over phase ids, origin at the bottom as imshow's
  ``origin="lower"``).
* ``save_checkpoint`` / ``load_checkpoint``: the packed compact state (heads
  plus the entries of cells that keep values) with everything a resume
  needs.  The reference keeps no restart state.
"""

from __future__ import annotations

import ctypes
import dataclasses
import json
import math
import struct
import zlib

import numpy as np

from . import _lib
from .inputs import Physics

FORMAT = "mpf3d-compact-checkpoint-1"
AXES = {"xy": 0, "xz": 1, "yz": 2}

# matplotlib's "tab20" colour table (the category20 palette), RGB
TAB20 = np.array([
    (31, 119, 180), (174, 199, 232), (255, 127, 14), (255, 187, 120), (44, 160, 44), (152, 223, 138),
    (214, 39, 40), (255, 152, 150), (148, 103, 189), (197, 176, 213), (140, 86, 75), (196, 156, 148),
    (227, 119, 194), (247, 182, 210), (127, 127, 127), (199, 199, 199), (188, 189, 34), (219, 219, 141),
    (23, 190, 207), (158, 218, 229)], np.uint8)


def _torch():
    import torch

    return torch


def _state(solver):
    h, i, v = solver.buf[solver.cur]
    return h.data_ptr(), i.data_ptr(), v.data_ptr()


# -- metrics ------------------------------------------------------------------------
def _run_metrics(solver, threshold: float):
    torch = _torch()
    res = torch.zeros(ctypes.sizeof(_lib.Metrics), dtype=torch.uint8, device=solver.device)
    gs = torch.zeros(solver.N, dtype=torch.float64, device=solver.device)
    front = torch.empty(solver.nx * solver.ny, dtype=torch.float32, device=solver.device)
    rc = _lib.lib().mpf3d_compact_metrics(*_state(solver), solver.slots, solver.N, solver.nx, solver.ny, solver.nz,
                                          float(threshold), res.data_ptr(), gs.data_ptr(), front.data_ptr(),
                                          solver._stream())
    _lib.check(rc, "compact_metrics")
    m = _lib.Metrics.from_buffer_copy(res.cpu().numpy().tobytes())
    return m, gs.cpu().numpy(), front


def metrics(solver, threshold: float = 0.5, runtime_s: float = 0.0) -> dict:
    """The dictionary of compute_metrics_3d (same keys and units) for the
    solver's current state."""
    m, gs, _ = _run_metrics(solver, threshold)
    dx = float(solver.phys.dx)
    v3 = dx ** 3
    grain_volumes = [float(g * v3) for g in gs[1:]]
    cols = int(m.front_columns)
    if cols:
        mean = m.front_sum / cols
        std = math.sqrt(max(m.front_sq_sum / cols - mean * mean, 0.0))
        mean_z, std_z, max_z = mean * dx, std * dx, m.front_max * dx
    else:
        mean_z = std_z = max_z = float("nan")
    nan = float("nan")
    return {
        "phi_sum_error_max": float(m.sum_err_max),
        "phi_min": float(m.phi_min),
        "phi_max": float(m.phi_max),
        "nf_max": int(m.nf_max),
        "nan_count": int(m.nan_count),
        "solid_fraction": float(m.solid_sum / solver.cells),
        "solid_volume": float(m.solid_sum * v3),
        "grain_volumes": grain_volumes,
        "surviving_grains": int(sum(v > v3 for v in grain_volumes)),
        "interface_position_mean": float(mean_z),
        "interface_position_max": float(max_z),
        "interface_position_std": float(std_z),
        "interface_roughness": float(std_z),
        "interface_angle_deg": nan,
        "solid_volume_growth": nan,
        "winner_loser_volume_ratio": nan,
        "grain_boundary_root_shift": nan,
        "trijunction_x": nan,
        "trijunction_z": nan,
        "dihedral_angle_like_metric": nan,
        "angle_deviation_from_final_state": nan,
        "front_velocity": nan,
        "runtime_s": float(runtime_s),
    }


def interface_positions(solver, threshold: float = 0.5) -> np.ndarray:
    """Highest z (cells) whose solid fraction exceeds `threshold`, per column:
    float64 [nx, ny], NaN where a column holds none."""
    _, _, front = _run_metrics(solver, threshold)
    return front.cpu().numpy().reshape(solver.ny, solver.nx).T.astype(np.float64)


# -- slices -----------------------------------------------------------------------------
def resolve_slice_index(axis: str, shape, index=None) -> int:
    """Default and clipping of the slice index (plot_utils_3d._resolve_slice_index)."""
    nx, ny, nz = shape
    if axis not in AXES:
        raise ValueError(f"Unsupported slice axis: {axis}")
    upper = {"xy": nz, "xz": ny, "yz": nx}[axis] - 1
    if index is None:
        return (upper + 1) // 2
    return int(np.clip(index, 0, upper))


def phase_slice(solver, axis: str = "xy", index=None) -> dict:
    """One slice of the current state: ``ids`` (argmax phase, int32),
    ``fraction`` (its value) and ``solid`` (1 - phi_liquid), each [W, H] with
    (W, H) = (nx, ny) for "xy", (nx, nz) for "xz", (ny, nz) for "yz"."""
    torch = _torch()
    idx = resolve_slice_index(axis, (solver.nx, solver.ny, solver.nz), index)
    W = solver.ny if axis == "yz" else solver.nx
    H = solver.ny if axis == "xy" else solver.nz
    ids = torch.empty(W * H, dtype=torch.int32, device=solver.device)
    frac = torch.empty(W * H, dtype=torch.float32, device=solver.device)
    solid = torch.empty(W * H, dtype=torch.float32, device=solver.device)
    rc = _lib.lib().mpf3d_compact_slice(*_state(solver), solver.slots, solver.nx, solver.ny, solver.nz, AXES[axis],
                                        idx, ids.data_ptr(), frac.data_ptr(), solid.data_ptr(), solver._stream())
    _lib.check(rc, "compact_slice")
    sh = (W, H)
    return {"axis": axis, "index": idx, "ids": ids.cpu().numpy().reshape(sh),
            "fraction": frac.cpu().numpy().reshape(sh), "solid": solid.cpu().numpy().reshape(sh)}


def write_png(path: str, rgb: np.ndarray) -> None:
    """8-bit RGB PNG (rows top to bottom) with zlib from the standard library."""
    rgb = np.ascontiguousarray(rgb, np.uint8)
    if rgb.ndim != 3 or rgb.shape[2] != 3:
        raise ValueError("rgb must be [H, W, 3] uint8")
    h, w, _ = rgb.shape
    raw = b"".join(b"\x00" + rgb[r].tobytes() for r in range(h))

    def chunk(tag: bytes, data: bytes) -> bytes:
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)

    with open(path, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n")
        f.write(chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 2, 0, 0, 0)))
        f.write(chunk(b"IDAT", zlib.compress(raw, 6)))
        f.write(chunk(b"IEND", b""))


def phase_colours(ids: np.ndarray, number_of_grain: int) -> np.ndarray:
    """tab20 colours of phase ids scaled over [0, number_of_grain - 1], as
    imshow(cmap="tab20", vmin=0, vmax=max(N - 1, 1)) colours them."""
    vmax = max(number_of_grain - 1, 1)
    k = np.clip((np.asarray(ids, np.float64) / vmax * 20.0).astype(np.int64), 0, 19)
    return TAB20[k]


def save_phase_map_png(path: str, sl: dict, number_of_grain: int, scale: int = 1) -> None:
    """PNG of a phase_slice: first slice axis to the right, second upwards."""
    img = phase_colours(sl["ids"].T[::-1], number_of_grain)
    if scale > 1:
        img = np.repeat(np.repeat(img, scale, axis=0), scale, axis=1)
    write_png(path, img)


# -- checkpoints --------------------------------------------------------------------------
def save_checkpoint(solver, path: str) -> dict:
    """Pack the state on the GPU and write it with the run's set-up to `path`
    (numpy .npz).  Returns {"entries", "bytes"}."""
    torch = _torch()
    L = _lib.lib()
    h, i, v = solver.buf[solver.cur]
    scratch = torch.empty(int(L.mpf3d_compact_pack_scratch_len(solver.cells)), dtype=torch.int64,
                          device=solver.device)
    total = torch.zeros(1, dtype=torch.int64, device=solver.device)
    st = solver._stream()
    rc = L.mpf3d_compact_pack(h.data_ptr(), i.data_ptr(), v.data_ptr(), solver.slots, solver.cells,
                              scratch.data_ptr(), total.data_ptr(), None, None, 0, solver.err.data_ptr(), st)
    _lib.check(rc, "compact_pack (count)")
    E = int(total.item())
    ids = torch.empty(max(E, 1), dtype=torch.int16, device=solver.device)
    vals = torch.empty(max(E, 1), dtype=torch.float32, device=solver.device)
    rc = L.mpf3d_compact_pack(h.data_ptr(), i.data_ptr(), v.data_ptr(), solver.slots, solver.cells,
                              scratch.data_ptr(), total.data_ptr(), ids.data_ptr(), vals.data_ptr(), E,
                              solver.err.data_ptr(), st)
    _lib.check(rc, "compact_pack")
    solver.check()
    t = solver.tuning
    arrays = dict(
        format=np.array(FORMAT),
        dims=np.array([solver.N, solver.nx, solver.ny, solver.nz], np.int64),
        slots=np.int64(solver.slots), step_count=np.int64(solver.step_count),
        head=h.cpu().numpy().view(np.uint32), ids=ids[:E].cpu().numpy().view(np.uint16),
        vals=vals[:E].cpu().numpy(),
        T_melt=np.float64(solver.T_melt), cooling_rate=np.float64(solver.cooling_rate),
        scalars=np.array(list(solver.scalars.v), np.float64), scalars_f32mask=np.int64(solver.scalars.f32mask),
        anisotropy=np.int64(solver.anisotropy), torque=np.int64(solver.torque),
        T0z=solver.T0z.cpu().numpy(), wij=solver.wij.cpu().numpy(), a2ij=solver.a2ij.cpu().numpy(),
        mij=solver.mij.cpu().numpy(), n111=solver.n111.cpu().numpy(),
        phys=np.array(json.dumps(dataclasses.asdict(solver.phys))),
        tuning=np.array([] if t is None else [t.sweep_zb, t.sweep_by, t.general_blocks_per_sm, t.general_threads,
                                              t.iface_blocks_per_sm, t.iface_threads], np.int64),
    )
    with open(path, "wb") as f:
        np.savez(f, **arrays)
    return {"entries": E, "bytes": int(sum(a.nbytes for a in arrays.values()))}


def load_checkpoint(cls, path: str, device="cuda:0", slots=None):
    """Rebuild a solver from `save_checkpoint` output; `slots` (optional)
    picks the slot template, which must hold the widest saved cell."""
    torch = _torch()
    from .solver import _SLOT_TEMPLATES

    d = np.load(path, allow_pickle=False)
    if str(d["format"]) != FORMAT:
        raise ValueError(f"{path} is not a {FORMAT} file")
    obj = cls.__new__(cls)
    obj.phys = Physics(**json.loads(str(d["phys"])))
    sc = _lib.Scalars()
    for k, x in enumerate(d["scalars"]):
        sc.v[k] = float(x)
    sc.f32mask = int(d["scalars_f32mask"])
    obj.scalars = sc
    obj.T_melt, obj.cooling_rate = float(d["T_melt"]), float(d["cooling_rate"])
    obj.anisotropy, obj.torque = bool(d["anisotropy"]), bool(d["torque"])
    obj.device = torch.device(device)
    obj.N, obj.nx, obj.ny, obj.nz = (int(x) for x in d["dims"])
    head = np.ascontiguousarray(d["head"], np.uint32)
    if head.size != obj.nx * obj.ny * obj.nz:
        raise ValueError("checkpoint head array does not match its dims")
    widest = int((head & 0x7F).max()) if head.size else 1
    want = int(slots if slots is not None else d["slots"])
    if want not in _SLOT_TEMPLATES:
        raise ValueError("slots must be 4, 8 or 16")
    while widest > want and want < max(_SLOT_TEMPLATES):
        want *= 2
    if widest > want:
        raise ValueError(f"a saved cell holds {widest} phases, above every slot template")
    obj._setup(want, d["T0z"], d["wij"], d["a2ij"], d["mij"], d["n111"])
    h, i_, v = obj.buf[0]
    h.copy_(torch.from_numpy(head.view(np.int32)).to(obj.device))
    E = int(d["ids"].size)
    ids = torch.from_numpy(np.ascontiguousarray(d["ids"]).view(np.int16)).to(obj.device) if E else \
        torch.zeros(1, dtype=torch.int16, device=obj.device)
    vals = torch.from_numpy(np.ascontiguousarray(d["vals"], np.float32)).to(obj.device) if E else \
        torch.zeros(1, dtype=torch.float32, device=obj.device)
    L = _lib.lib()
    scratch = torch.empty(int(L.mpf3d_compact_pack_scratch_len(obj.cells)), dtype=torch.int64, device=obj.device)
    rc = L.mpf3d_compact_unpack(h.data_ptr(), ids.data_ptr(), vals.data_ptr(), E, obj.slots, obj.cells,
                                scratch.data_ptr(), i_.data_ptr(), v.data_ptr(), obj.err.data_ptr(), obj._stream())
    _lib.check(rc, "compact_unpack")
    obj.step_count = int(d["step_count"])
    obj.check()
    if d["tuning"].size == 6:
        t = _lib.Tuning()
        (t.sweep_zb, t.sweep_by, t.general_blocks_per_sm, t.general_threads, t.iface_blocks_per_sm,
         t.iface_threads) = (int(x) for x in d["tuning"])
        obj.tuning = t
    return obj
