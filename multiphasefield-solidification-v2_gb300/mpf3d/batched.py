"""Batched bicrystals: hundreds of independent 3D domains of uneven size in
one set of step launches, replayed from a CUDA graph.

Replaces the reference's one-domain-at-a-time loops
(run_orientation_scan_3d.py:686-841; the bicrystal runs of
tests/verification_3d.py:1951-2011) with a single batched engine: every
instance is a vertical grain boundary splitting a solid base into grain 1
(x < nx/2) and grain 2, under its own uniform undercooling, anisotropy
strength and pair of orientations.  The observables -- front height of each
grain half, grain volumes and the grain-boundary crossing rows -- are reduced
on the GPU; only per-instance numbers come back to the host.
"""

from __future__ import annotations

import ctypes
import math

import numpy as np

from . import _lib
from .inputs import Physics, interaction_matrices, rotated_n111

TILE = (32, 8, 4)  # sweep tile of the step kernels (x, y, z)
_SLOT_TEMPLATES = {4: 8, 8: 16, 16: 32}


class Instance(ctypes.Structure):
    """mpf3d_instance (include/mpf3d.h)."""
    _fields_ = [("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32),
                ("offset", ctypes.c_uint32), ("n111_base", ctypes.c_int32), ("split", ctypes.c_int32),
                ("tile_start", ctypes.c_int32), ("delta_a", ctypes.c_float), ("mu_da", ctypes.c_float),
                ("e2_flat", ctypes.c_float), ("undercooling", ctypes.c_float),
                ("base_height", ctypes.c_float)]


def _e2_flat(phys: Physics, delta_a: float) -> float:
    """(eps0 a)^2 at a vanishing liquid gradient, as the single-domain step computes it."""
    d = phys.derived()
    pp = phys.p_round * phys.p_round
    a = phys.mu_a * (1.0 + delta_a * (math.sqrt(pp) + math.tan(d["a0"]) * math.sqrt(1.0 + pp)))
    e = d["eps0_sl"] * a
    return float(np.float32(e * e))


class BatchedBicrystals:
    """A batch of independent domains stepped together.  layout="bicrystal"
    (default): grain 1 | grain 2 over a base of `base_height` cells, liquid
    above.  layout="sphere": a sphere of grain 1 with radius[i] cells centred
    at center[i] (cells; default the box centre nx/2, ny/2, nz/2) in liquid,
    the set-up of the reference's orientation scan (grain 2 stays absent)."""

    def __init__(self, dims, quats, undercooling, delta_a, phys: Physics | None = None, *,
                 base_height: float = 16.0, slots: int = 4, anisotropy: bool = True,
                 torque: bool = True, device="cuda:0", layout: str = "bicrystal", radius=None,
                 center=None):
        import torch

        self.torch = torch
        self.phys = phys or Physics()
        self.device = torch.device(device)
        self.dims = [tuple(int(v) for v in d) for d in dims]
        n = len(self.dims)
        if n == 0:
            raise ValueError("empty batch")
        quats = np.asarray(quats, np.float64)
        if quats.shape != (n, 2, 4):
            raise ValueError("quats must be [n_instances, 2, 4] (x, y, z, w) for grains 1 and 2")
        self.undercooling = np.asarray(undercooling, np.float64).reshape(n)
        self.delta_a = np.asarray(delta_a, np.float64).reshape(n)
        if slots not in _SLOT_TEMPLATES:
            raise ValueError("slots must be 4, 8 or 16")
        self.slots, self.amax = slots, _SLOT_TEMPLATES[slots]
        self.anisotropy, self.torque = bool(anisotropy), bool(torque)
        self.base_height = float(base_height)

        d = self.phys.derived()
        insts = (Instance * n)()
        off = tile = 0
        row_base = []
        rows = 0
        for i, (nx, ny, nz) in enumerate(self.dims):
            I = insts[i]
            I.nx, I.ny, I.nz = nx, ny, nz
            I.offset = off
            I.n111_base = 3 * i
            I.split = nx // 2
            I.tile_start = tile
            da = float(self.delta_a[i])
            I.delta_a = da
            I.mu_da = float(np.float32(self.phys.mu_a * da))
            I.e2_flat = _e2_flat(self.phys, da)
            I.undercooling = float(self.undercooling[i])
            I.base_height = self.base_height
            off += nx * ny * nz
            tile += -(-nx // TILE[0]) * -(-ny // TILE[1]) * -(-nz // TILE[2])
            row_base.append(rows)
            rows += nz
        if off >= 2 ** 31:
            raise ValueError("batch holds 2^31 cells or more")
        self.n, self.total_cells, self.n_tiles = n, off, tile
        self.inst_host = insts
        self.inst = torch.frombuffer(bytearray(bytes(insts)), dtype=torch.uint8).to(self.device)
        self.row_base = torch.tensor(row_base, dtype=torch.int32, device=self.device)
        self.rows_total = rows

        full_q = np.zeros((3 * n, 4))
        full_q[0::3] = (0.0, 0.0, 0.0, 1.0)
        full_q[1::3] = quats[:, 0]
        full_q[2::3] = quats[:, 1]
        n111 = rotated_n111(full_q)
        self.symmetric_normals = bool(np.array_equal(n111[:, 4:8], -n111[:, [3, 2, 1, 0]]))
        wij, aij, mij = interaction_matrices(3, d["eps0_sl"], d["w0_sl"], d["m_sl_phi"], d["eps_gb"],
                                             d["w_gb"], d["m_gb_phi"])
        to = lambda a: torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float32).to(self.device)
        self.n111, self.wij, self.a2ij, self.mij = to(n111), to(wij), to(aij * aij), to(mij)
        self.scalars = _lib.Scalars()
        for k, v in enumerate(self.phys.kernel_scalars(f32=False)):
            self.scalars.v[k] = float(v)
        self.err = torch.zeros(1, dtype=torch.int32, device=self.device)
        # the three work lists of MPF3D_STEP_MULTI_LIST and their counters
        self.work_items = torch.empty(2 * self.total_cells, dtype=torch.int32, device=self.device)
        self.work_count = torch.zeros(6, dtype=torch.int32, device=self.device)
        # quiet-tile flags of the batched sweep (zero: the next step visits every tile)
        n_flags = int(_lib.lib().mpf3d_batched_tile_flags_len(self.n_tiles))
        self.tile_flags = torch.zeros(max(n_flags, 1), dtype=torch.uint8, device=self.device)
        self.skip_quiet_tiles = True
        self.buf = [self._alloc(), self._alloc()]
        self.cur = 0
        self.step_count = 0
        self.graph = None
        self.tuning = None  # work-list kernel shape (mpf3d_tuning); None = library default
        h, i_, v = self.buf[0]
        self.layout = layout
        if layout == "bicrystal":
            rc = _lib.lib().mpf3d_batched_init_bicrystal(self._ip(), n, self.total_cells, self.phys.dx,
                                                         d["delta"], h.data_ptr(), i_.data_ptr(),
                                                         v.data_ptr(), self.err.data_ptr(), self._stream())
            _lib.check(rc, "batched_init_bicrystal")
        elif layout == "sphere":
            if radius is None:
                raise ValueError("layout='sphere' needs radius (cells, scalar or per instance)")
            rad = np.array(np.broadcast_to(np.asarray(radius, np.float64), (n,)))
            if center is None:
                cen = np.array([[nx / 2.0, ny / 2.0, nz / 2.0] for nx, ny, nz in self.dims])
            else:
                cen = np.array(np.broadcast_to(np.asarray(center, np.float64), (n, 3)))
            self.center_cells = np.ascontiguousarray(cen, np.float64)
            self.radius_cells = np.ascontiguousarray(rad, np.float64)
            self._center = torch.as_tensor(self.center_cells, dtype=torch.float32).to(self.device)
            self._radius = torch.as_tensor(self.radius_cells, dtype=torch.float32).to(self.device)
            rc = _lib.lib().mpf3d_batched_init_sphere(self._ip(), n, self.total_cells, self.phys.dx, d["delta"],
                                                      self._center.data_ptr(), self._radius.data_ptr(), 1,
                                                      self.slots, h.data_ptr(), i_.data_ptr(), v.data_ptr(),
                                                      self._stream())
            _lib.check(rc, "batched_init_sphere")
        else:
            raise ValueError(f"unknown layout {layout!r}")
        self.check()

    # -- plumbing ----------------------------------------------------------------
    def _alloc(self):
        t = self.torch
        return (t.empty(self.total_cells, dtype=t.int32, device=self.device),
                t.empty(self.slots * self.total_cells, dtype=t.int16, device=self.device),
                t.empty(self.slots * self.total_cells, dtype=t.float32, device=self.device))

    def _ip(self):
        return self.inst.data_ptr()

    def _stream(self):
        return self.torch.cuda.current_stream(self.device).cuda_stream or None

    def check(self):
        v = int(self.err.item())
        if v:
            self.err.zero_()
            raise RuntimeError("batched solver device error: " + _lib.describe_dev_error(v))

    # -- stepping ----------------------------------------------------------------
    def launch_step(self) -> None:
        src, dst = self.buf[self.cur], self.buf[1 - self.cur]
        self.step_count += 1
        rc = _lib.lib().mpf3d_batched_step_tuned(
            src[0].data_ptr(), src[1].data_ptr(), src[2].data_ptr(), dst[0].data_ptr(), dst[1].data_ptr(),
            dst[2].data_ptr(), self.slots, self.amax, self._ip(), self.n, self.n_tiles, self.total_cells,
            self.wij.data_ptr(), self.a2ij.data_ptr(), self.mij.data_ptr(), self.n111.data_ptr(), 3,
            ctypes.byref(self.scalars), int(self.anisotropy), int(self.torque), int(self.symmetric_normals),
            self.work_items.data_ptr(), self.work_count.data_ptr(), self.step_count & 1,
            self.err.data_ptr(), self._stream(), _lib.STEP_MULTI_LIST,
            ctypes.byref(self.tuning) if self.tuning is not None else None,
            self.tile_flags.data_ptr() if self.skip_quiet_tiles else None)
        _lib.check(rc, "batched_step")
        self.cur = 1 - self.cur

    def forget_history(self) -> None:
        """Clear what the step keeps from earlier steps -- the quiet-tile flags
        and the work-list counters.  Required after the state buffers are
        written other than by a step (restore); the next step then visits
        every tile."""
        self.tile_flags.zero_()
        self.work_count.zero_()

    def autotune(self, steps: int = 8, use_cache: bool = True) -> dict:
        """Pick the fastest work-list kernel shape for this batch (see
        mpf3d.autotune.tune_batched); call before capture()."""
        from . import autotune

        return autotune.tune_batched(self, steps=steps, use_cache=use_cache)

    def capture(self, steps: int):
        """Capture `steps` (even) consecutive steps in a CUDA graph."""
        t = self.torch
        if steps % 2:
            raise ValueError("capture an even number of steps so the buffers and parities line up")
        s = t.cuda.Stream(self.device)
        s.wait_stream(t.cuda.current_stream(self.device))
        g = t.cuda.CUDAGraph()
        cur0, count0 = self.cur, self.step_count
        with t.cuda.graph(g, stream=s):
            for _ in range(steps):
                self.launch_step()
        # capture recorded the launches without running them
        self.cur, self.step_count = cur0, count0
        t.cuda.current_stream(self.device).wait_stream(s)
        self.graph, self.graph_steps = g, steps

    def step(self, n: int, use_graph: bool = True) -> None:
        n = int(n)
        if use_graph and self.graph is not None:
            while n >= self.graph_steps:
                self.graph.replay()
                self.step_count += self.graph_steps
                n -= self.graph_steps
        for _ in range(n):
            self.launch_step()

    # -- observables ---------------------------------------------------------------
    def fronts(self):
        """Per instance: (mean front height left, right) in cells and (sum phi1, sum phi2)."""
        t = self.torch
        acc = t.zeros(6 * self.n, dtype=t.float64, device=self.device)
        h, i_, v = self.buf[self.cur]
        rc = _lib.lib().mpf3d_batched_fronts(h.data_ptr(), i_.data_ptr(), v.data_ptr(), self.slots, self._ip(),
                                             self.n, self.total_cells, acc.data_ptr(), self._stream())
        _lib.check(rc, "batched_fronts")
        a = acc.view(self.n, 6).cpu().numpy()
        with np.errstate(invalid="ignore", divide="ignore"):
            return a[:, 0] / a[:, 1], a[:, 2] / a[:, 3], a[:, 4], a[:, 5]

    def gb_inclination(self, z_from=None, z_margin: float = 2.0):
        """Per instance: grain-boundary inclination in degrees from vertical
        (positive: the boundary leans towards grain 2, i.e. grain 1 widens with
        height) from a least-squares fit of the y-averaged phi1 = phi2
        crossing x(z) over the rows from the initial base height up to the
        lower front minus `z_margin`."""
        t = self.torch
        gb = t.zeros(2 * self.rows_total, dtype=t.float64, device=self.device)
        h, i_, v = self.buf[self.cur]
        rc = _lib.lib().mpf3d_batched_gb_rows(h.data_ptr(), i_.data_ptr(), v.data_ptr(), self.slots, self._ip(),
                                              self.n, self.total_cells, self.row_base.data_ptr(),
                                              gb.data_ptr(), self._stream())
        _lib.check(rc, "batched_gb_rows")
        rows = gb.view(self.rows_total, 2).cpu().numpy()
        hl, hr, _, _ = self.fronts()
        z0 = self.base_height if z_from is None else z_from
        out = np.full(self.n, np.nan)
        base = 0
        for i, (nx, ny, nz) in enumerate(self.dims):
            r = rows[base:base + nz]
            base += nz
            top = min(hl[i], hr[i]) - z_margin
            ks = np.arange(nz, dtype=np.float64)
            sel = (r[:, 1] > 0) & (ks >= z0) & (ks <= top)
            if sel.sum() >= 6:
                xs = r[sel, 0] / r[sel, 1]
                slope = np.polyfit(ks[sel], xs, 1)[0]
                out[i] = math.degrees(math.atan(slope))
        return out

    def ray_radii(self, dirs, threshold: float = 0.5, step_cells: float = 0.5, phase: int = 1,
                  center=None) -> np.ndarray:
        """directional_radius_symmetric (run_orientation_scan_3d.py:338-351)
        of `phase` from each instance's centre along each direction: the mean
        of the finite crossing distances (cells) along +d and -d, NaN if
        neither crosses.  Returns [n_instances, n_dirs]."""
        t = self.torch
        dirs = np.ascontiguousarray(np.asarray(dirs, np.float64).reshape(-1, 3))
        if center is None:
            if not hasattr(self, "_center"):
                raise ValueError("center is needed for layouts without a sphere centre")
            cen = self._center
        else:
            cen = t.as_tensor(np.broadcast_to(np.asarray(center, np.float64), (self.n, 3)).copy(),
                              dtype=t.float32).to(self.device)
        dd = t.as_tensor(dirs, dtype=t.float32).to(self.device)
        out = t.empty(self.n * len(dirs) * 2, dtype=t.float64, device=self.device)
        h, i_, v = self.buf[self.cur]
        rc = _lib.lib().mpf3d_batched_ray_radii(h.data_ptr(), i_.data_ptr(), v.data_ptr(), self.slots, self._ip(),
                                                self.n, self.total_cells, int(phase), cen.data_ptr(), dd.data_ptr(),
                                                len(dirs), float(threshold), float(step_cells), out.data_ptr(),
                                                self._stream())
        _lib.check(rc, "batched_ray_radii")
        r = out.view(self.n, len(dirs), 2).cpu().numpy()
        with np.errstate(invalid="ignore"):
            fin = np.isfinite(r)
            cnt = fin.sum(axis=2)
            mean = np.where(fin, r, 0.0).sum(axis=2) / np.maximum(cnt, 1)
        return np.where(cnt > 0, mean, np.nan)

    def dense(self, i: int, dtype=np.float32):
        """Dense phi [3, nx, ny, nz] of instance i (host)."""
        t = self.torch
        nx, ny, nz = self.dims[i]
        out = t.empty((3, nx, ny, nz), dtype=t.float32 if dtype == np.float32 else t.float64, device=self.device)
        h, i_, v = self.buf[self.cur]
        rc = _lib.lib().mpf3d_compact_to_dense_view(h.data_ptr(), i_.data_ptr(), v.data_ptr(), self.slots,
                                                    self.total_cells, self.inst_host[i].offset, 3, nx, ny, nz,
                                                    out.data_ptr(), 0 if dtype == np.float32 else 1,
                                                    self._stream())
        _lib.check(rc, "compact_to_dense_view")
        return out.cpu().numpy()

    def run(self, steps: int, sample_every: int = 50, graph_steps: int = 50):
        """Advance `steps` steps, sampling the fronts and grain volumes every
        `sample_every` steps.  Per instance, each grain's growth velocity
        (cells/step) is the slope of its volume divided by its footprint
        (its half of the base), fitted over the samples taken while both
        fronts stay 6 cells below the top; returns the velocities, their ratio
        (grain 1 / grain 2) and the final grain-boundary inclination."""
        if self.graph is None and graph_steps:
            self.capture(graph_steps)
        times, h1, h2, V1, V2 = [0], [], [], [], []

        def sample():
            a, b, v1, v2 = self.fronts()
            h1.append(a)
            h2.append(b)
            V1.append(v1)
            V2.append(v2)

        sample()
        done = 0
        while done < steps:
            k = min(sample_every, steps - done)
            self.step(k)
            done += k
            times.append(done)
            sample()
        self.check()
        times = np.asarray(times, np.float64)
        H1, H2, A1, A2 = (np.stack(x, 1) for x in (h1, h2, V1, V2))
        v1 = np.full(self.n, np.nan)
        v2 = np.full(self.n, np.nan)
        for i, (nx, ny, nz) in enumerate(self.dims):
            ok = (H1[i] < nz - 6) & (H2[i] < nz - 6)
            if ok.sum() >= 2:
                split = nx // 2
                v1[i] = np.polyfit(times[ok], A1[i, ok], 1)[0] / (split * ny)
                v2[i] = np.polyfit(times[ok], A2[i, ok], 1)[0] / ((nx - split) * ny)
        with np.errstate(invalid="ignore", divide="ignore"):
            ratio = v1 / v2
        # why a ratio is not finite: 1 = fewer than two samples before a front
        # came within 6 cells of the top (fast growth in a short box), 2 =
        # grain 2 does not grow (zero fitted velocity)
        status = np.zeros(self.n, np.int32)
        status[~np.isfinite(v1) | ~np.isfinite(v2)] = 1
        status[(status == 0) & (v2 == 0.0)] = 2
        status[(status == 0) & ~np.isfinite(ratio)] = 3
        return {"v1": v1, "v2": v2, "velocity_ratio": ratio, "gb_angle_deg": self.gb_inclination(),
                "times": times, "h1": H1, "h2": H2, "V1": A1, "V2": A2, "ratio_status": status}


def sample_batch(n: int, seed: int = 0, sizes_xy=(64, 96, 128), sizes_z=(64, 96), dT_range=(0.25, 3.0),
                 delta_a_range=(0.0, 1.0)):
    """Instance parameters of the batched-bicrystal workload: grid sizes drawn
    uniformly from sizes_xy^2 x sizes_z, uniform random orientation pairs,
    undercooling and anisotropy strength uniform in their ranges."""
    rng = np.random.default_rng(seed)
    dims = [(int(rng.choice(sizes_xy)), int(rng.choice(sizes_xy)), int(rng.choice(sizes_z))) for _ in range(n)]
    q = rng.standard_normal((n, 2, 4))
    q /= np.linalg.norm(q, axis=2, keepdims=True)
    dT = rng.uniform(*dT_range, n)
    da = rng.uniform(*delta_a_range, n)
    return dims, q, dT, da
