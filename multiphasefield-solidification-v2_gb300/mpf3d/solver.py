"""Compact FP32 solver: the fused one-kernel-per-step tier.

``CompactSolver`` owns a double-buffered compact state on one GPU (see
include/mpf3d.h for the layout) and advances it with ``mpf3d_compact_step``.
It replaces the reference's driver loop (run_randommode_3d.py:267-287:
temperature kernel, APT kernel, update kernel, buffer swap) with one launch
per step; dense phi is only materialised on request (``to_dense``).

Device memory comes from torch (plumbing only); all compute is in
libmpf3d.so.
"""

from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .inputs import Physics

_SLOT_TEMPLATES = {4: 8, 8: 16, 16: 32}  # slots -> max active phases per cell


class _DenseShape:
    """Shape-only stand-in for a dense phi that is never formed."""

    def __init__(self, N, nx, ny, nz):
        self.shape = (N, nx, ny, nz)


class SlotOverflow(RuntimeError):
    """A cell needed more slots (or active phases) than the template holds."""


def _torch():
    import torch

    return torch


def _scalars_from(phys_or_tuple):
    s = _lib.Scalars()
    if isinstance(phys_or_tuple, Physics):
        vals = phys_or_tuple.kernel_scalars(f32=False)
    else:
        vals = phys_or_tuple
    if len(vals) != 13:
        raise ValueError("13 kernel scalars expected")
    for i, v in enumerate(vals):
        s.v[i] = float(v)
    s.f32mask = 0
    return s


def z_profile(temp) -> np.ndarray:
    """Temperature as a float64 z profile; 3-D fields must be uniform in x, y."""
    t = np.asarray(temp, dtype=np.float64)
    if t.ndim == 1:
        return np.ascontiguousarray(t)
    if t.ndim != 3:
        raise ValueError("temperature must be [nz] or [nx, ny, nz]")
    prof = t[0, 0, :]
    if not np.array_equal(t, np.broadcast_to(prof, t.shape)):
        raise ValueError("the compact tier takes a temperature that depends on z only")
    return np.ascontiguousarray(prof)


class CompactSolver:
    """Compact FP32 stepper of one domain.  Build it from a dense phi0 or, for
    domains whose dense field does not fit, with `from_owner`."""

    def __init__(self, phi0, temp0, n111, wij, aij, mij, phys: Physics | None = None, *,
                 scalars=None, T_melt=None, cooling_rate=None, slots: int = 8,
                 anisotropy: bool = True, torque: bool = True, device="cuda:0"):
        torch = _torch()
        if slots not in _SLOT_TEMPLATES:
            raise ValueError(f"slots must be one of {sorted(_SLOT_TEMPLATES)}")
        owner_init = None
        if isinstance(phi0, tuple) and len(phi0) == 3 and phi0[0] == "owner":
            owner_init = phi0[1]
            phi0 = _DenseShape(*phi0[2])
        self.phys = phys or Physics()
        d = self.phys.derived()
        self.scalars = _scalars_from(scalars if scalars is not None else self.phys)
        self.T_melt = float(self.phys.T_melt if T_melt is None else T_melt)
        self.cooling_rate = float(d["cooling_rate"] if cooling_rate is None else cooling_rate)
        self.anisotropy, self.torque = bool(anisotropy), bool(torque)
        self.device = torch.device(device)
        if owner_init is not None:
            phi = phi0
        else:
            phi = phi0 if isinstance(phi0, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(phi0))
            if phi.dim() != 4 or phi.dtype not in (torch.float32, torch.float64):
                raise ValueError("phi0 must be float32/float64 [N, nx, ny, nz]")
        self.N, self.nx, self.ny, self.nz = (int(s) for s in phi.shape)
        if tuple(np.shape(aij)) != (self.N, self.N):
            raise ValueError(f"aij must have shape {(self.N, self.N)}")
        aij32 = np.asarray(aij, np.float32)
        self._setup(slots, z_profile(temp0), wij, aij32 * aij32, mij, n111)
        if owner_init is not None:
            owner, slab, prof = owner_init
            h, i_, v = self.buf[0]
            rc = _lib.lib().mpf3d_compact_init_owner(owner.data_ptr(), slab, prof.data_ptr(), self.nx, self.ny,
                                                     self.nz, self.slots, h.data_ptr(), i_.data_ptr(),
                                                     v.data_ptr(), self._stream())
            _lib.check(rc, "compact_init_owner")
        elif phi.device.type == "cpu" and phi.is_pinned() and phi.is_contiguous():
            # pinned host memory: the converter reads it in place over the
            # CPU-GPU link (no device copy of the dense field)
            self._from_dense(phi, _lib.host_device_pointer(phi))
        else:
            dphi = phi.to(self.device).contiguous()
            self._from_dense(dphi)
        self.check()

    def _setup(self, slots, t0z, wij, a2ij, mij, n111):
        """Device-side set-up shared by the constructors: matrices, scratch and
        the two state buffers (contents undefined)."""
        torch = _torch()
        self.cells = self.nx * self.ny * self.nz
        self.slots = slots
        self.amax = _SLOT_TEMPLATES[slots]
        to = lambda a, dt: torch.as_tensor(np.ascontiguousarray(a), dtype=dt).to(self.device)
        self.T0z = to(t0z, torch.float64)
        if self.T0z.numel() != self.nz:
            raise ValueError("temperature profile length must equal nz")
        for nm, a, shp in (("wij", wij, (self.N, self.N)), ("a2ij", a2ij, (self.N, self.N)),
                           ("mij", mij, (self.N, self.N)), ("n111", n111, (self.N, 8, 3))):
            if tuple(np.shape(a)) != shp:
                raise ValueError(f"{nm} must have shape {shp}")
        self.wij = to(np.asarray(wij, np.float32), torch.float32)
        self.a2ij = to(np.asarray(a2ij, np.float32), torch.float32)
        self.mij = to(np.asarray(mij, np.float32), torch.float32)
        self.n111 = to(np.asarray(n111, np.float32), torch.float32)
        self.err = torch.zeros(1, dtype=torch.int32, device=self.device)
        # scratch of the step: the three work lists (MPF3D_STEP_MULTI_LIST) and their counters
        self.work_items = torch.empty(2 * self.cells, dtype=torch.int32, device=self.device)
        self.work_count = torch.zeros(6, dtype=torch.int32, device=self.device)
        n111_np = np.asarray(n111, np.float32)
        self.symmetric_normals = bool(np.array_equal(n111_np[:, 4:8], -n111_np[:, [3, 2, 1, 0]]))
        self.buf = [self._alloc(), self._alloc()]
        self.cur = 0
        self.step_count = 0
        self.tuning = None  # launch shape (mpf3d_tuning); None = library default
        # quiet-tile flags of the sweep (see mpf3d_compact_step_tuned)
        self.skip_quiet_tiles = True
        # the sweep stages its heads in shared memory by TMA (same results)
        self.sweep_tma = False
        n_flags = int(_lib.lib().mpf3d_compact_tile_flags_len(self.nx, self.ny, self.nz))
        self.tile_flags = torch.zeros(max(n_flags, 1), dtype=torch.uint8, device=self.device)
        self._tiles_zb = None
        # device step clock (mpf3d_step_clock: int64 step[2], float64 tmc[2])
        # and the step index it holds for the next step (None: unknown)
        self.clock = torch.zeros(4, dtype=torch.int64, device=self.device)
        self._clock_next = None
        self.graph = None  # CUDA graph of captured steps (capture())

    def forget_history(self) -> None:
        """Clear what the step keeps from earlier steps -- the quiet-tile flags
        and the work-list counters.  Required after the state buffers are
        written other than by a step (restore, rollback); the next step then
        visits every tile."""
        self.tile_flags.zero_()
        self.work_count.zero_()

    @classmethod
    def from_owner(cls, owner, profile, temp0, n111, wij, aij, mij, phys: Physics | None = None, **kw):
        """Start from a grain-owner map of the first `slab` z-layers (int32
        [nx, ny, slab], grains 1..N-1; higher layers repeat the top one) and a
        solid-fraction z profile, without forming the dense field."""
        torch = _torch()
        own = np.asarray(owner)
        nx, ny, slab = own.shape
        nz = len(profile)
        N = int(np.asarray(wij).shape[0])
        dev = torch.device(kw.get("device", "cuda:0"))
        o = torch.as_tensor(np.ascontiguousarray(own.transpose(2, 1, 0)), dtype=torch.int32).to(dev)
        p = torch.as_tensor(np.ascontiguousarray(profile, np.float32)).to(dev)
        return cls(("owner", (o, slab, p), (N, nx, ny, nz)), temp0, n111, wij, aij, mij, phys, **kw)

    # -- buffers ---------------------------------------------------------------
    def _alloc(self):
        torch = _torch()
        return (torch.empty(self.cells, dtype=torch.int32, device=self.device),
                torch.empty(self.slots * self.cells, dtype=torch.int16, device=self.device),
                torch.empty(self.slots * self.cells, dtype=torch.float32, device=self.device))

    def _stream(self):
        return _torch().cuda.current_stream(self.device).cuda_stream or None

    def _from_dense(self, dphi, ptr=None):
        torch = _torch()
        cnt, idx, val = self.buf[self.cur]
        rc = _lib.lib().mpf3d_compact_from_dense(
            dphi.data_ptr() if ptr is None else ptr, 0 if dphi.dtype == torch.float32 else 1, self.N, self.nx, self.ny,
            self.nz, self.slots, cnt.data_ptr(), idx.data_ptr(), val.data_ptr(),
            self.err.data_ptr(), self._stream())
        _lib.check(rc, "compact_from_dense")

    # -- stepping ---------------------------------------------------------------
    def launch_step(self, step_index: int) -> None:
        """Enqueue one step (no synchronisation); step_index is 1-based.

        The step runs at T_melt + step_index * cooling_rate, which it reads
        from the solver's device clock (mpf3d_compact_step_clocked); the clock
        is set here only when step_index is not the step that follows the
        last one launched.  Only the parity is passed by value, so a CUDA
        graph of an even number of consecutive steps (capture()) can be
        replayed over and over and keeps cooling."""
        src = self.buf[self.cur]
        dst = self.buf[1 - self.cur]
        zb = self.tuning.sweep_zb if self.tuning is not None else 4
        if zb != self._tiles_zb:  # the tile geometry follows the sweep shape
            self.tile_flags.zero_()
            self._tiles_zb = zb
        if step_index != self._clock_next:
            self.clock[step_index & 1].fill_(step_index)  # a kernel: no host copy, capturable
        rc = _lib.lib().mpf3d_compact_step_clocked(
            src[0].data_ptr(), src[1].data_ptr(), src[2].data_ptr(), dst[0].data_ptr(),
            dst[1].data_ptr(), dst[2].data_ptr(), self.slots, self.amax, self.T0z.data_ptr(),
            self.clock.data_ptr(), self.T_melt, self.cooling_rate,
            self.wij.data_ptr(), self.a2ij.data_ptr(), self.mij.data_ptr(), self.n111.data_ptr(),
            self.N, self.nx, self.ny, self.nz, ctypes.byref(self.scalars), int(self.anisotropy),
            int(self.torque), int(self.symmetric_normals), self.work_items.data_ptr(),
            self.work_count.data_ptr(), step_index & 1, self.err.data_ptr(), self._stream(),
            ctypes.byref(self.tuning) if self.tuning is not None else None,
            self.tile_flags.data_ptr() if self.skip_quiet_tiles else None,
            _lib.STEP_MULTI_LIST | (_lib.STEP_SWEEP_TMA if self.sweep_tma else 0))
        _lib.check(rc, "compact_step")
        self._clock_next = step_index + 1
        self.cur = 1 - self.cur

    def capture(self, steps: int) -> None:
        """Capture `steps` (even) consecutive steps, starting at the next one,
        in a CUDA graph; step() then replays it wherever it fits (same
        buffers and parity) and launches the rest one by one.  Capture after
        autotune() and after setting sweep_tma / skip_quiet_tiles: the graph
        keeps the launch shape it was captured with."""
        torch = _torch()
        steps = int(steps)
        if steps <= 0 or steps % 2:
            raise ValueError("capture an even number of steps so the buffers and parities line up")
        n0 = self.step_count + 1
        zb = self.tuning.sweep_zb if self.tuning is not None else 4
        if zb != self._tiles_zb:
            self.tile_flags.zero_()
            self._tiles_zb = zb
        if self._clock_next != n0:  # set outside the graph: a replay must not reset it
            self.clock[n0 & 1].fill_(n0)
            self._clock_next = n0
        cs = torch.cuda.Stream(self.device)
        cs.wait_stream(torch.cuda.current_stream(self.device))
        _lib.check(_lib.lib().mpf3d_streams_prepare(cs.cuda_stream), "streams_prepare")
        g = torch.cuda.CUDAGraph()
        cur0 = self.cur
        with torch.cuda.graph(g, stream=cs):
            for i in range(steps):
                self.launch_step(n0 + i)
        torch.cuda.current_stream(self.device).wait_stream(cs)
        # the capture recorded the steps without running them
        self.cur, self._clock_next = cur0, n0
        self.graph, self.graph_steps, self._graph_at = g, steps, (cur0, n0 & 1, self.buf[cur0][0].data_ptr())

    def _advance(self, n: int) -> None:
        """Launch n steps: graph replays where the captured graph fits, the
        rest one by one."""
        while n > 0:
            g = self.graph
            if (g is not None and n >= self.graph_steps and
                    self._graph_at == (self.cur, (self.step_count + 1) & 1, self.buf[self.cur][0].data_ptr())):
                if self._clock_next != self.step_count + 1:
                    self.clock[(self.step_count + 1) & 1].fill_(self.step_count + 1)
                g.replay()
                self.step_count += self.graph_steps
                self._clock_next = self.step_count + 1
                n -= self.graph_steps
            else:
                self.step_count += 1
                self.launch_step(self.step_count)
                n -= 1

    def step(self, n: int = 1, check: bool = True, check_every: int = 200) -> None:
        """Advance n steps (replaying the graph of capture() where it fits).
        With check=True the device error word is read every `check_every`
        steps; a slot overflow rolls the state back to the start of that
        chunk, widens the slot template (4 -> 8 -> 16) and redoes the chunk,
        so no phase is ever dropped silently."""
        n = int(n)
        if not check:
            self._advance(n)
            return
        done = 0
        while done < n:
            chunk = min(int(check_every), n - done)
            ckpt = [t.clone() for t in self.buf[self.cur]], self.step_count
            self._advance(chunk)
            v = int(self.err.item())
            if v & 8 and self.slots < max(_SLOT_TEMPLATES):
                self.err.zero_()
                self._restore_widened(ckpt)
                continue
            self.check()
            done += chunk

    def _restore_widened(self, ckpt) -> None:
        (cnt, idx, val), steps = ckpt
        old = self.slots
        self.slots = {4: 8, 8: 16}[old]
        self.amax = _SLOT_TEMPLATES[self.slots]
        self.buf = [self._alloc(), self._alloc()]
        self.cur = 0
        c2, i2, v2 = self.buf[0]
        c2.copy_(cnt)
        i2[: old * self.cells].copy_(idx)
        v2[: old * self.cells].copy_(val)
        self.step_count = steps
        self.graph = None  # captured for the old buffers
        self.forget_history()

    def autotune(self, steps: int = 8, use_cache: bool = True) -> dict:
        """Pick the fastest launch shape for this problem (see mpf3d.autotune)."""
        from . import autotune

        return autotune.tune(self, steps=steps, use_cache=use_cache)

    def check(self) -> None:
        v = int(self.err.item())
        if v:
            self.err.zero_()
            msg = _lib.describe_dev_error(v)
            if v & 8:
                raise SlotOverflow(f"compact state overflow ({msg}); use more slots")
            raise RuntimeError(f"compact solver device error: {msg}")

    # -- outputs ----------------------------------------------------------------
    def to_dense(self, dtype=np.float32, host: bool = True, out=None):
        """Dense phi [N, nx, ny, nz].  With `out` (a contiguous tensor of that
        shape and of dtype float32 or float64) the field is written there
        and `out` is returned: a pinned CPU tensor is written in place over
        the CPU-GPU link, asynchronously on the solver's stream (synchronise
        before reading it)."""
        torch = _torch()
        shape = (self.N, self.nx, self.ny, self.nz)
        if out is not None:
            if tuple(out.shape) != shape or out.dtype not in (torch.float32, torch.float64) or not out.is_contiguous():
                raise ValueError(f"out must be a contiguous float32/float64 tensor of shape {shape}")
            tdt = out.dtype
            if out.device.type == "cpu":
                if not out.is_pinned():
                    raise ValueError("a CPU `out` must be pinned (page-locked)")
                ptr = _lib.host_device_pointer(out)
            else:
                ptr = out.data_ptr()
        else:
            tdt = torch.float32 if np.dtype(dtype) == np.float32 else torch.float64
            out = torch.empty(shape, dtype=tdt, device=self.device)
            ptr = out.data_ptr()
        cnt, idx, val = self.buf[self.cur]
        rc = _lib.lib().mpf3d_compact_to_dense(cnt.data_ptr(), idx.data_ptr(), val.data_ptr(),
                                               self.slots, self.N, self.nx, self.ny, self.nz,
                                               ptr, 0 if tdt == torch.float32 else 1, self._stream())
        _lib.check(rc, "compact_to_dense")
        if out.device.type == "cpu":
            return out
        return out.cpu().numpy() if host else out

    def active_count(self, host: bool = True):
        torch = _torch()
        nf = torch.empty((self.nx, self.ny, self.nz), dtype=torch.int32, device=self.device)
        cnt, idx, _ = self.buf[self.cur]
        rc = _lib.lib().mpf3d_compact_active_count(cnt.data_ptr(), idx.data_ptr(), self.slots,
                                                   self.nx, self.ny, self.nz, nf.data_ptr(),
                                                   self._stream())
        _lib.check(rc, "compact_active_count")
        return nf.cpu().numpy() if host else nf

    def stored_counts(self):
        """Number of stored phases per cell (x-fastest order)."""
        return self.buf[self.cur][0] & 0x7F

    def record_bytes(self) -> int:
        """Bytes of the current state that a step must read: the 4-byte head
        of every cell plus 6 bytes per stored phase of cells holding two or
        more (4 for an explicitly stored single value)."""
        h = self.buf[self.cur][0]
        n = (h & 0x7F).long()
        e = ((h >> 7) & 1).long()
        extra = _torch().where(n >= 2, 6 * n - 2, 4 * e)
        return int(4 * self.cells + extra.sum().item())

    def state_bytes(self) -> int:
        return self.cells * (4 + 6 * self.slots)

    # -- observables and checkpoints (computed on the GPU, see mpf3d.observe) ----
    def metrics(self, threshold: float = 0.5, runtime_s: float = 0.0) -> dict:
        """compute_metrics_3d (tests/verification_3d.py:612-654) of the current state."""
        from . import observe

        return observe.metrics(self, threshold=threshold, runtime_s=runtime_s)

    def interface_positions(self, threshold: float = 0.5) -> np.ndarray:
        """interface_positions_3d (tests/verification_3d.py:409-416): [nx, ny] float64, NaN where no solid."""
        from . import observe

        return observe.interface_positions(self, threshold=threshold)

    def phase_slice(self, axis: str = "xy", index=None) -> dict:
        """Argmax phase ids, their fractions and the solid fraction of one slice."""
        from . import observe

        return observe.phase_slice(self, axis=axis, index=index)

    def save(self, path: str) -> dict:
        """Write a checkpoint (.npz) of the state and everything a resume needs."""
        from . import observe

        return observe.save_checkpoint(self, path)

    @classmethod
    def load(cls, path: str, device="cuda:0", slots=None) -> "CompactSolver":
        """Resume from a checkpoint written by `save`; the next step continues
        the run exactly."""
        from . import observe

        return observe.load_checkpoint(cls, path, device=device, slots=slots)
