"""Benchmark of the 3D multi-phase-field step on GB300.

Workload (default): 256^3 grid, 64 grains seeded uniformly in the bottom 32
z-layers (3D Voronoi) plus liquid (N = 65 phases), tanh front, anisotropy and
torque on, uniform cooling, config_3d.yaml physics, 2000 steps -- advanced by
the compact FP32 stepper (sweep, general and interface kernels per step).
Synthetic seeded inputs of the configured shape; no dataset is involved.

With --gpus N (one process per GPU under torchrun) every rank advances its own
replica of the workload and its own share of the bicrystal batch: the work is
independent, no data crosses ranks, and the timings are the maximum over ranks
(weak scaling).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  `value` is cell-steps/s with the state
resident in HBM; `e2e` runs the same job through the public API from pinned
host memory (dense phi in, dense phi out) with the copies timed.  The
reference arm (--impl reference) times the CPU oracle -- a C restatement of
the reference kernels with their float32 typing -- on all host cores over a
bounded crop of the same workload.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "multiphasefield-solidification-v2_gb300")
for p in (PKG, ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)

METRIC = "3D cell-steps/s (FP32 compact step, 256^3, N=65)"
UNIT = "cell-steps/s"
GRID = (256, 256, 256)
N_GRAINS = 64
SLAB = 32
SEED, ORIENT_SEED = 2026, 7
FALLBACK_BF16_TFLOPS = 1900.0
FALLBACK_HBM_GBS = 6800.0


def workload_owner(nx, ny, nz):
    from mpf3d import inputs
    return inputs.voronoi_slab_owner(nx, ny, nz, N_GRAINS, SLAB, SEED)


def workload_inputs(phys):
    from mpf3d import inputs
    q = inputs.random_quaternions(N_GRAINS, ORIENT_SEED)
    wij, aij, mij = inputs.matrices_for(phys, N_GRAINS + 1)
    return inputs.rotated_n111(q), wij, aij, mij


def dense_phi_on_device(owner_t, prof_t, torch):
    """Dense phi [N, nx, ny, nz] built on the GPU from the owner map."""
    nx, ny, nz = owner_t.shape
    phi = torch.zeros((N_GRAINS + 1, nx, ny, nz), dtype=torch.float32, device=owner_t.device)
    solid = prof_t.view(1, 1, nz).expand(nx, ny, nz)
    phi.scatter_(0, owner_t.long().unsqueeze(0), solid.unsqueeze(0).contiguous())
    phi[0] = torch.clamp(1.0 - phi[1:].sum(dim=0), 0.0, 1.0)
    return phi


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            time.sleep(0.15)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return None
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "samples": len(sm),
                "reasons": sorted(reasons)}


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM_GBS, "fallback"


def gemm_run(dev, M=65536, N=256, K=256, reps=20):
    """The surrogate's hidden-layer GEMM (Y = SiLU(X W^T + b), BF16 in, FP32
    accumulate, BF16 out) at the screening batch: the tcgen05 kernel and the
    mma.sync kernel, timed with CUDA events, against the measured dense BF16
    peak (burst: the kernel is timed alone)."""
    import torch
    from mpf3d import _lib
    L = _lib.lib()
    g = torch.Generator(device="cpu").manual_seed(5)
    X = (torch.randn((M, K), generator=g) * 0.5).to(torch.bfloat16).to(dev)
    W = (torch.randn((N, K), generator=g) * 0.06).to(torch.bfloat16).to(dev)
    b = torch.zeros(N, dtype=torch.float32, device=dev)
    Y = torch.empty((M, N), dtype=torch.bfloat16, device=dev)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    st = torch.cuda.current_stream(dev)
    calls = {
        "tc5": lambda: L.mpf3d_gemm_bf16_tc5(M, N, K, X.data_ptr(), K, W.data_ptr(), K, b.data_ptr(), 1, None,
                                             Y.data_ptr(), N, 1, 0, err.data_ptr(), st.cuda_stream or None),
        "mma": lambda: L.mpf3d_gemm_bf16_mma(M, N, K, X.data_ptr(), K, 1, W.data_ptr(), 1, K, b.data_ptr(), 1, None,
                                             Y.data_ptr(), N, 1, 0, st.cuda_stream or None),
    }
    out = {"shape": [M, N, K], "flop": 2.0 * M * N * K}
    for name, fn in calls.items():
        for _ in range(3):
            assert fn() == 0
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(dev)
        e0.record(st)
        for _ in range(reps):
            fn()
        e1.record(st)
        torch.cuda.synchronize(dev)
        us = e0.elapsed_time(e1) * 1e3 / reps
        out[f"{name}_us"] = us
        out[f"{name}_tflops"] = out["flop"] / (us * 1e-6) / 1e12
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peak = float(json.load(f)["bf16_tflops"])
        out["peak_bf16_tflops"], out["peak_source"] = peak, "measured (burst)"
    except (OSError, KeyError, ValueError):
        peak = FALLBACK_BF16_TFLOPS
        out["peak_bf16_tflops"], out["peak_source"] = peak, "fallback"
    if int(err.item()):
        raise RuntimeError("tcgen05 GEMM aborted: " + _lib.describe_dev_error(int(err.item())))
    out["tc5_frac"] = out["tc5_tflops"] / peak
    out["mma_frac"] = out["mma_tflops"] / peak
    return out


def cell_record_bytes(solver):
    """Bytes of every cell's record (int64 [cells], x fastest): the 4-byte
    head plus 6 bytes per stored phase of cells holding two or more (4 for
    an explicitly stored single value)."""
    import torch
    h = solver.buf[solver.cur][0]
    n = (h & 0x7F).long()
    e = ((h >> 7) & 1).long()
    return 4 + torch.where(n >= 2, 6 * n - 2, 4 * e)


def quiet_cells(solver, step_index):
    """Cells (bool [cells], x fastest) in the tiles that the step
    `step_index` skips: tiles that were uniform, with their 6 neighbours, in
    the previous step (the rule of the sweep kernel)."""
    import torch
    zb = solver.tuning.sweep_zb if solver.tuning is not None else 4
    nx, ny, nz = solver.nx, solver.ny, solver.nz
    ntx, nkb = -(-nx // 32), -(-nz // zb)
    n = nkb * ny * ntx
    if not solver.skip_quiet_tiles or solver._tiles_zb != zb:
        return torch.zeros(solver.cells, dtype=torch.bool, device=solver.device)
    half = (step_index & 1) ^ 1
    f = solver.tile_flags[half * n:(half + 1) * n].view(nkb, ny, ntx).bool()
    q = f & torch.roll(f, 1, 2) & torch.roll(f, -1, 2) & torch.roll(f, 1, 1) & torch.roll(f, -1, 1)
    q = q & torch.cat([f[1:], f[-1:]], 0) & torch.cat([f[:1], f[:-1]], 0)
    q = q.repeat_interleave(zb, 0)[:nz].repeat_interleave(32, 2)[:, :, :nx]
    return q.reshape(-1)


def committed_traffic():
    """DRAM bytes per step of the three step kernels over the bench's timed
    steps 1-20, from the committed ncu summary (a 128 x 128 x 256 crop with the
    same grain density, one kernel per capture, scaled 4x to 256^3 by area)."""
    path = os.path.join(ROOT, "profiles", "compact_step_dram_crop128x128x256_steps1-20.md")
    try:
        for line in open(path):
            if line.startswith("dram_bytes_per_step_256cube_scaled:"):
                return float(line.split(":", 1)[1].split()[0])
    except OSError:
        pass
    return None


def cpu_oracle_rate(phys, cx, cy, seconds, max_steps=None, warmup=0):
    """Oracle (reference typing: float32 phi and scalars) on a cx x cy x 256
    crop of the workload; returns (cell-steps/s, steps, cells, threads)."""
    import oracle as O
    from mpf3d import inputs
    nz = GRID[2]
    owner = workload_owner(GRID[0], GRID[1], nz)[:cx, :cy, :].copy()
    d = phys.derived()
    prof = inputs.tanh_profile(nz, SLAB, phys.dx, d["delta"])
    phi = inputs.phi_from_owner(owner, N_GRAINS, prof)
    temp = inputs.temperature_field(cx, cy, nz, phys.T_melt, phys.G, phys.dx, SLAB)
    n111, wij, aij, mij = workload_inputs(phys)
    sc = O.make_scalars([float(v) for v in phys.kernel_scalars(True)], True)
    rate = d["cooling_rate"]
    phi_new = phi.copy()
    mf = np.zeros((50, cx, cy, nz), np.int32)
    nf = np.zeros((cx, cy, nz), np.int32)

    def one():
        nonlocal phi, phi_new
        O.temp_step(temp, rate, True)
        st = np.zeros(2, np.int32)
        O.apt(phi, mf, nf, st, checked=True)
        O.update(phi, phi_new, temp, mf, nf, wij, aij, mij, n111, sc, switchable=False)
        phi, phi_new = phi_new, phi

    for _ in range(warmup):
        one()
    t0 = time.perf_counter()
    steps = 0
    while True:
        one()
        steps += 1
        el = time.perf_counter() - t0
        if (max_steps is not None and steps >= max_steps) or (max_steps is None and el >= seconds):
            break
    cells = cx * cy * nz
    threads = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return cells * steps / el, steps, cells, threads


def run_reference(args, rank):
    if rank != 0:
        return
    from mpf3d.inputs import Physics
    phys = Physics()
    total = args.steps + args.warmup
    # crop sized so that the whole run stays within about two minutes
    side = 64 if total <= 60 else (32 if total <= 400 else 16)
    val, steps, cells, threads = cpu_oracle_rate(phys, side, side, 0.0, max_steps=args.steps,
                                                 warmup=args.warmup)
    sample = f"{side}x{side}x256 crop of the workload (N=65), {steps} oracle steps"
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 storage, f64/f32 reference typing",
            "data": "synthetic", "config": config_dict(args),
            "cpu_baseline": {"value": val, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def config_dict(args):
    nx, ny, nz = GRID
    return {"workload": f"3D random Voronoi {nx}x{ny}x{nz}, {N_GRAINS} grains in the bottom {SLAB} z-layers + "
                        f"liquid (N={N_GRAINS + 1}), tanh front, anisotropy+torque on, uniform cooling "
                        "(config_3d.yaml), FP32 compact three-kernel step",
            "grid": list(GRID), "phases": N_GRAINS + 1, "slots": args.slots, "steps": args.steps,
            "l2": "inputs larger than L2, no flush: the two state buffers' head arrays alone are "
                  "2 x 67 MB (> 129 MB L2), plus the stored records; each step reads the previous "
                  "step's output",
            "parallelism": f"replicas x{args.gpus}" if args.gpus > 1 else "single GPU"}


def run_ours(args, rank, world):
    import torch
    from mpf3d import inputs
    from mpf3d.solver import CompactSolver

    local = int(os.environ.get("LOCAL_RANK", "0"))
    dev = torch.device(f"cuda:{local}")
    torch.cuda.set_device(dev)
    phys = inputs.Physics()
    d = phys.derived()
    nx, ny, nz = GRID
    owner = torch.from_numpy(workload_owner(nx, ny, nz)).to(dev)
    prof = torch.from_numpy(inputs.tanh_profile(nz, SLAB, phys.dx, d["delta"])).to(dev)
    temp = inputs.temperature_field(1, 1, nz, phys.T_melt, phys.G, phys.dx, SLAB)[0, 0]
    n111, wij, aij, mij = workload_inputs(phys)
    phi0 = dense_phi_on_device(owner, prof, torch)
    solver = CompactSolver(phi0, temp, n111, wij, aij, mij, phys, slots=args.slots)
    stream = torch.cuda.current_stream(dev)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    # warm-up (including the launch-shape search), then restart the job from
    # the initial state with the chosen shape
    solver.step(args.warmup)
    tuned = solver.autotune(steps=8) if not args.no_autotune else None
    torch.cuda.synchronize(dev)
    tuning, sweep_tma = solver.tuning, solver.sweep_tma
    solver = CompactSolver(phi0, temp, n111, wij, aij, mij, phys, slots=args.slots)
    solver.tuning, solver.sweep_tma = tuning, sweep_tma
    # the timed steps are captured once into a CUDA graph (their temperatures
    # come from the solver's device clock) and replayed in the timed region;
    # an odd step count runs eagerly
    use_graph = args.steps % 2 == 0 and not args.no_graph
    if use_graph:
        solver.capture(args.steps)
    torch.cuda.synchronize(dev)

    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier()
        torch.cuda.synchronize(dev)
        e0.record(stream)
        solver.step(args.steps, check=False)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        barrier()
    solver.check()
    ms = max_over_ranks(e0.elapsed_time(e1), world)
    final_cnt_sum = int(solver.stored_counts().sum(dtype=torch.int64).item())

    # accounting pass (untimed), the same run again: per step, the record
    # bytes of the cells the step visits (read of the old record, write of
    # the new one; cells of tiles skipped as quiet move nothing), the quiet
    # share and the stored-phase occupancy
    acc = CompactSolver(phi0, temp, n111, wij, aij, mij, phys, slots=args.slots)
    acc.tuning, acc.sweep_tma = tuning, sweep_tma
    occ = [int(acc.stored_counts().sum(dtype=torch.int64).item())]
    rec_all = 0
    bytes_total = 0
    quiet_share = 0.0
    r_prev = cell_record_bytes(acc)
    for i in range(args.steps):
        skip = quiet_cells(acc, i + 1)
        acc.launch_step(i + 1)
        r_next = cell_record_bytes(acc)
        both = r_prev + r_next
        rec_all += int(both.sum().item())
        bytes_total += int(both[~skip].sum().item())
        quiet_share += float(skip.float().mean().item())
        occ.append(int(acc.stored_counts().sum(dtype=torch.int64).item()))
        r_prev = r_next
    acc.check()
    del acc
    cells = nx * ny * nz
    # algorithmic bytes: every visited cell's record read once and written once
    bytes_per_launch = bytes_total / args.steps
    full_state_bytes = rec_all / args.steps
    quiet_share /= args.steps
    sec = ms / 1e3
    value = cells * args.steps * world / sec
    per_launch_s = sec / args.steps
    peak, peak_kind = measured_peak()
    achieved = bytes_per_launch / per_launch_s / 1e9
    traffic = committed_traffic()

    # end to end through the public API: pinned dense phi in, dense phi out
    if args.no_e2e:
        t_e2e, in_bytes, out_bytes, t_staged = float("nan"), 0, 0, float("nan")
    else:
        t_e2e, in_bytes, out_bytes, t_staged = e2e_run(args, phi0, temp, n111, wij, aij, mij, phys, dev, barrier,
                                                       world, tuning, sweep_tma)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        v, st, cl, th = cpu_oracle_rate(phys, 64, 64, 10.0)
        cpu = {"value": v, "unit": UNIT, "cores": th, "kind": "port",
               "sample": f"64x64x256 crop of the workload (N=65), {st} oracle steps (reference "
                         f"float32 typing), OpenMP"}
    extra = {"e2e_staged_copies": {"value": cells * args.steps * world / t_staged, "unit": UNIT,
                                   "note": "the same job with dense phi copied to device memory and back "
                                           "(cudaMemcpy of pinned buffers) instead of converted in place"},
             "launch_shape": {"config": list(tuned["config"]), "sweep_tma": bool(sweep_tma),
                              "ms_per_step_tuned": tuned["ms_per_step"],
                              "ms_per_step_default": tuned["default_ms_per_step"]} if tuned else None,
             "timed_steps_from": "one CUDA graph of the timed steps, replayed once (temperatures from the "
                                 "solver's device step clock)" if use_graph else "eager launches"}
    if rank == 0 and not args.no_accuracy and args.accuracy_steps > 0:
        del solver
        torch.cuda.empty_cache()
        extra["accuracy_fp32_vs_fp64"] = accuracy_run(args, phi0, temp, n111, wij, aij, mij, phys, dev)
        extra["accuracy_fp32_vs_fp64"]["groove_and_bicrystal"] = groove_accuracy(dev)
    if rank == 0 and not args.no_dense_reference:
        extra["reference_numerics_dense_gb300"] = dense_reference_rate(phi0, temp, n111, wij, aij, mij, phys, dev)
    del phi0
    torch.cuda.empty_cache()
    if not args.no_bicrystal and args.bicrystal_steps > 0:
        extra["bicrystal_batch"] = bicrystal_run(args, dev, rank, world)
    if rank == 0 and not args.no_gemm:
        extra["surrogate_gemm"] = gemm_run(dev)
    emit(args, rank, world, value, ms, cells, t_e2e, in_bytes, out_bytes, achieved, peak, peak_kind,
         traffic, bytes_per_launch, occ, clk, cpu, final_cnt_sum, dict(extra, quiet_tile_share=quiet_share,
                                                                         full_state_bytes_per_cell_step=
                                                                         full_state_bytes / cells))


def e2e_run(args, phi0, temp, n111, wij, aij, mij, phys, dev, barrier, world, tuning=None, sweep_tma=False):
    import torch
    from mpf3d.solver import CompactSolver
    phi_host = phi0.cpu().pin_memory()
    out_host = torch.empty_like(phi_host).pin_memory()

    def job(steps, staged=False):
        if staged:
            # staging copies: dense phi copied to device memory and back
            dphi = phi_host.to(dev, non_blocking=True)
            s2 = CompactSolver(dphi, temp, n111, wij, aij, mij, phys, slots=args.slots)
        else:
            # the converters read and write the pinned host buffers in place
            s2 = CompactSolver(phi_host, temp, n111, wij, aij, mij, phys, slots=args.slots)
        s2.tuning, s2.sweep_tma = tuning, sweep_tma
        s2.step(steps, check=False)
        if staged:
            out_host.copy_(s2.to_dense(host=False), non_blocking=True)
        else:
            s2.to_dense(out=out_host)
        return s2

    times = {}
    for staged in (False, True):
        # untimed warm-up pass of the same sequence: the first 4.4 GB device
        # allocations of a process cost a box-dependent 20-70 ms that a user
        # submitting jobs pays once; the timed pass keeps every copy
        job(args.warmup, staged).check()
        torch.cuda.synchronize(dev)
        barrier()
        t0 = time.perf_counter()
        s2 = job(args.steps, staged)
        torch.cuda.synchronize(dev)
        times[staged] = time.perf_counter() - t0
        s2.check()
        del s2
        barrier()
    t_e2e = max_over_ranks(times[False], world)
    in_bytes = phi_host.numel() * 4 + temp.nbytes + n111.nbytes + 3 * wij.nbytes
    out_bytes = out_host.numel() * 4
    return t_e2e, in_bytes, out_bytes, max_over_ranks(times[True], world)


def dense_reference_rate(phi0, temp, n111, wij, aij, mij, phys, dev, steps=20):
    """The same 256^3 workload on the drop-in kernels: the reference's own
    algorithm, dense [N][nx][ny][nz] layout and float32 typing, in the step
    sequence of run_randommode_3d.py:267-287 (temperature, APT, update,
    swap), timed with CUDA events.  The reference's Numba kernels cannot run
    where numba is absent; this is the same arithmetic on the same GPU."""
    import torch
    from src import gpu_kernels_3d as K
    N, nx, ny, nz = phi0.shape
    p = phi0.clone()
    q = torch.empty_like(p)
    T = torch.from_numpy(np.ascontiguousarray(np.broadcast_to(np.asarray(temp, np.float32), (nx, ny, nz)))).to(dev)
    mf = torch.zeros((50, nx, ny, nz), dtype=torch.int32, device=dev)
    nf = torch.zeros((nx, ny, nz), dtype=torch.int32, device=dev)
    W, A, M, U = (torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in (wij, aij, mij, n111))
    sc = phys.kernel_scalars(f32=True)
    rate = np.float32(phys.derived()["cooling_rate"])
    cfg = ((-(-nx // 4), -(-ny // 4), -(-nz // 4)), (4, 4, 4))
    stream = torch.cuda.current_stream(dev)

    def step():
        nonlocal p, q
        K.kernel_update_temp_3d[cfg](T, rate, nx, ny, nz)
        K.kernel_update_nfmf_3d[cfg](p, mf, nf, nx, ny, nz, N)
        K.kernel_update_phasefield_active_3d[cfg](p, q, T, mf, nf, W, A, M, U, nx, ny, nz, N, *sc)
        p, q = q, p

    for _ in range(3):
        step()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(dev)
    e0.record(stream)
    for _ in range(steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize(dev)
    K.check_errors()
    ms = e0.elapsed_time(e1) / steps
    out = {"cell_steps_per_s": nx * ny * nz / (ms * 1e-3), "ms_per_step": ms, "steps": steps,
           "kernels": "drop-in src/gpu_kernels_3d.py: temperature, APT, kernel_update_phasefield_active_3d",
           "typing": "float32 phi and scalars, float64 arithmetic (the reference's compiled-Numba typing)"}
    del p, q, T, mf, nf
    torch.cuda.empty_cache()
    return out


def _dense_run(phi0, temp_value, quats, phys, steps, aniso, torque, f64, dev):
    """The reference harness's step sequence on the drop-in kernels: FP64
    (float64 phi, temperature and scalars) or the reference's own float32
    typing."""
    import torch
    from mpf3d import inputs
    from src import gpu_kernels_3d as K
    N, nx, ny, nz = phi0.shape
    dt = np.float64 if f64 else np.float32
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    p, q = t(phi0.astype(dt)), t(phi0.astype(dt))
    T = t(np.full((nx, ny, nz), dt(temp_value), dt))
    mf = torch.zeros((50, nx, ny, nz), dtype=torch.int32, device=dev)
    nf = torch.zeros((nx, ny, nz), dtype=torch.int32, device=dev)
    wij, aij, mij = inputs.matrices_for(phys, N)
    W, A, M, U = t(wij), t(aij), t(mij), t(inputs.rotated_n111(quats))
    sc = phys.kernel_scalars(f32=not f64)
    rate = dt(phys.derived()["cooling_rate"])
    cfg = ((-(-nx // 4), -(-ny // 4), -(-nz // 4)), (4, 4, 4))
    for _ in range(steps):
        if float(rate) != 0.0:
            K.kernel_update_temp_3d[cfg](T, rate, nx, ny, nz)
        K.kernel_update_nfmf_3d[cfg](p, mf, nf, nx, ny, nz, N)
        K.kernel_update_phasefield_active_3d_switchable[cfg](p, q, T, mf, nf, W, A, M, U, nx, ny, nz, N, *sc,
                                                             np.int32(aniso), np.int32(torque))
        p, q = q, p
    torch.cuda.synchronize(dev)
    K.check_errors()
    return p.cpu().numpy()


def groove_accuracy(dev):
    """Groove and bicrystal observables (mpf3d.groove: the reference's
    robust_groove_metrics and bicrystal_group_metrics,
    tests/verification_3d.py:571-609, 1366-1381) of FP32 runs against FP64:
      groove     -- the groove_depth_only set-up (20x6x24 bicrystal, isotropic,
                    20 steps at T_melt, tests/verification_3d.py:2453-2488);
      bicrystal  -- the kinetic-regime set-up (18x6x28, aligned{111} | identity,
                    delta_a 0.35, ksi 0.01, 6 K undercooling, 10 steps,
                    :2326-2385)."""
    from scipy.spatial.transform import Rotation
    from mpf3d import groove, inputs
    from mpf3d.solver import CompactSolver
    lib = inputs.orientation_library()
    setups = {
        "groove": (inputs.Physics(delta_a=0.0, ksi=1.0, G=0.0, V_pulling=0.0), (20, 6, 24), 10, 0.6, 20,
                   0.0, inputs.quaternions_of([Rotation.identity()] * 2), 0),
        "bicrystal": (inputs.Physics(delta_a=0.35, ksi=0.01, p_round=0.02, G=0.0, V_pulling=0.0), (18, 6, 28), 9,
                      0.8, 10, 6.0, inputs.quaternions_of([lib["aligned_111_to_z"], lib["identity"]]), 1),
    }
    out = {}
    for name, (phys, (nx, ny, nz), split, wav, steps, dT, q, aniso) in setups.items():
        phi0 = inputs.bicrystal_field(nx, ny, nz, phys.dx, phys.derived()["delta"], 7.0, split, waviness=wav)
        root0 = groove.grain_boundary_root(phi0, 1, 2, x_guess=split)["root_x_cells"]
        T = phys.T_melt - dT
        runs = {"fp64": _dense_run(phi0, T, q, phys, steps, aniso, 0, True, dev),
                "f32_reference_numerics": _dense_run(phi0, T, q, phys, steps, aniso, 0, False, dev)}
        wij, aij, mij = inputs.matrices_for(phys, 3)
        c = CompactSolver(phi0, np.full(nz, T), inputs.rotated_n111(q), wij, aij, mij, phys,
                          anisotropy=bool(aniso), torque=False, device=dev)
        c.step(steps)
        runs["fp32_compact"] = c.to_dense(np.float32)
        rec = {}
        for k, phi in runs.items():
            gm = groove.groove_metrics(phi, root_x_guess=float(split))
            fam = groove.family_volumes(phi, [1], [2], phys.dx)
            rec[k] = {"dihedral_angle_like_deg": gm["dihedral_angle_like_deg"],
                      "root_z_cells": gm["root_z_cells"], "groove_depth_cells": gm["groove_depth_cells"],
                      "root_shift_cells": gm["root_x_cells"] - root0,
                      "winner_loser_volume_ratio": fam["winner_loser_volume_ratio"],
                      "max_abs_dphi_vs_fp64": float(np.abs(phi.astype(np.float64) - runs["fp64"]).max())}
        for k in ("f32_reference_numerics", "fp32_compact"):
            rec[k]["dihedral_diff_deg"] = rec[k]["dihedral_angle_like_deg"] - rec["fp64"]["dihedral_angle_like_deg"]
        out[name] = rec
    return out


def interface_height(phi_liquid):
    """Mean over columns of the highest z with solid fraction > 0.5
    (interface_positions_3d, tests/verification_3d.py:409-416)."""
    import torch
    solid = 1.0 - phi_liquid
    mask = solid > 0.5
    nz = mask.shape[-1]
    ks = torch.arange(nz, device=mask.device).view(1, 1, nz)
    top = torch.where(mask, ks, torch.full_like(ks, -1)).amax(dim=-1)
    ok = top >= 0
    return float(top[ok].double().mean().item()) if bool(ok.any()) else float("nan")


def divergence_study(phi0, temp, n111, wij, aij, mij, phys, dev, steps, slots=16, checkpoints=None,
                     every_step_until=100, seed=11):
    """Pointwise FP32-vs-FP64 error trajectories, every run stepped in
    lockstep on the GPU from the same float32 initial state (so no run starts
    with a rounding difference):
      reference (FP64)        -- the dense drop-in kernels with float64 phi,
                                 temperature and scalars (pinned to the
                                 oracle at 1e-12);
      fp32_compact            -- the FP32 compact stepper of the bench line;
      f32_reference_numerics  -- the reference's own production typing
                                 (float32 phi and scalars, float64 arithmetic);
      fp64_fp32_storage       -- exact FP64 arithmetic with phi rounded to
                                 float32 after every step: what storing the
                                 state in FP32 costs by itself;
      fp64_noise_1ulp         -- FP64 with a random relative perturbation of
                                 2^-52 (one float64 ulp) of every value in
                                 (0, 1) after every step.
    Per checkpoint and run: max|dphi| against FP64, cells above 1e-4 and
    1e-6, support flips (a (phase, cell) entry positive in one run and zero
    in the other), mean interface height and the largest grain
    volume-fraction difference.  Per run: the first step above 1e-4 and the
    first step with a support flip (checked every step up to
    every_step_until, then at the checkpoints)."""
    import torch
    from mpf3d.solver import CompactSolver
    from src import gpu_kernels_3d as K
    if checkpoints is None:
        checkpoints = (1, 10, 50, 100, 200, 500, 1000, 2000)
    ck = {c for c in checkpoints if c <= steps} | {steps}
    N, nx, ny, nz = phi0.shape
    cells = nx * ny * nz
    rate = phys.derived()["cooling_rate"]
    W, A, M, U = (torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in (wij, aij, mij, n111))
    T0 = np.broadcast_to(np.asarray(temp, np.float64), (nx, ny, nz))
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed)

    class Dense:
        def __init__(self, dtype, f32):
            self.p = phi0.to(dtype=dtype, copy=True).contiguous()
            self.q = torch.empty_like(self.p)
            self.T = torch.from_numpy(np.ascontiguousarray(T0, dtype=np.float32 if f32 else np.float64)).to(dev)
            self.mf = torch.zeros((50, nx, ny, nz), dtype=torch.int32, device=dev)
            self.nf = torch.zeros((nx, ny, nz), dtype=torch.int32, device=dev)
            self.sc = phys.kernel_scalars(f32=f32)
            self.rate = (np.float32 if f32 else np.float64)(rate)

        def step(self):
            cfg = ((1, 1, 1), (4, 4, 4))
            K.kernel_update_temp_3d[cfg](self.T, self.rate, nx, ny, nz)
            K.kernel_update_nfmf_3d[cfg](self.p, self.mf, self.nf, nx, ny, nz, N)
            K.kernel_update_phasefield_active_3d[cfg](self.p, self.q, self.T, self.mf, self.nf, W, A, M, U,
                                                      nx, ny, nz, N, *self.sc)
            self.p, self.q = self.q, self.p

    def noise_1ulp(p):
        r = torch.rand(p.shape, generator=gen, device=dev, dtype=torch.float32)
        inner = (p > 0) & (p < 1)
        # the factor 1 +- 2^-52 formed in float64 (a float32 scalar would round it to 1)
        factor = 1.0 + torch.where(r < 0.5, -1.0, 1.0).double() * 2.0 ** -52
        p.copy_(torch.where(inner, p * factor, p))

    ref = Dense(torch.float64, False)
    runs = {"f32_reference_numerics": Dense(torch.float32, True), "fp64_fp32_storage": Dense(torch.float64, False),
            "fp64_noise_1ulp": Dense(torch.float64, False)}
    comp = CompactSolver(phi0, temp, n111, wij, aij, mij, phys, slots=slots)
    names = ["fp32_compact"] + list(runs)
    first_above = {k: None for k in names}
    first_flip = {k: None for k in names}

    def summary(r, o, full):
        d = (r - o).abs().amax(dim=0)
        rec = {"max_abs_dphi": float(d.max().item()), "flips": int(((r > 0) != (o > 0)).sum().item())}
        if full:
            vf_r = r[1:].sum(dim=(1, 2, 3)) / cells
            vf_o = o[1:].sum(dim=(1, 2, 3)) / cells
            rec.update({"cells_above_1e-4": int((d > 1e-4).sum().item()),
                        "cells_above_1e-6": int((d > 1e-6).sum().item()),
                        "interface_height_cells": interface_height(o[0]),
                        "grain_volume_fraction_max_abs_diff": float((vf_r - vf_o).abs().max().item())})
        return rec

    traj = []
    t0 = time.perf_counter()
    for s in range(1, steps + 1):
        ref.step()
        for r in runs.values():
            r.step()
        runs["fp64_fp32_storage"].p.copy_(runs["fp64_fp32_storage"].p.float())
        noise_1ulp(runs["fp64_noise_1ulp"].p)
        comp.step(1, check=False)
        full = s in ck
        if not (full or s <= every_step_until):
            continue
        rp = ref.p
        rec = {"step": s}
        others = {"fp32_compact": comp.to_dense(host=False).double()}
        for k, r in runs.items():
            others[k] = r.p.double() if r.p.dtype != torch.float64 else r.p
        for k in names:
            rec[k] = summary(rp, others[k], full)
            if first_above[k] is None and rec[k]["max_abs_dphi"] > 1e-4:
                first_above[k] = s
            if first_flip[k] is None and rec[k]["flips"] > 0:
                first_flip[k] = s
        del others
        if full:
            rec["fp64_interface_height_cells"] = interface_height(rp[0])
            traj.append(rec)
    torch.cuda.synchronize(dev)
    comp.check()
    K.check_errors()
    out = {"steps": steps, "grid": [nx, ny, nz], "phases": N, "tolerance": 1e-4, "trajectory": traj,
           "first_step_above_tolerance": first_above, "first_step_with_support_flip": first_flip,
           "seconds": time.perf_counter() - t0,
           "note": "fp64_fp32_storage is exact FP64 arithmetic on a state rounded to float32 every step; "
                   "its divergence is what FP32 storage costs by itself"}
    del ref, runs, comp
    torch.cuda.empty_cache()
    return out


def accuracy_run(args, phi0, temp, n111, wij, aij, mij, phys, dev):
    """The divergence study of the bench workload over --accuracy-steps."""
    return divergence_study(phi0, temp, n111, wij, aij, mij, phys, dev, args.accuracy_steps, slots=args.slots)


def _reduce_scalar(x: float, world: int, op) -> float:
    if world <= 1:
        return float(x)
    import torch
    dist = torch.distributed
    # NCCL reduces device tensors only; gloo (the CPU tests) host tensors
    dev = (torch.device("cuda", torch.cuda.current_device())
           if dist.get_backend() == "nccl" else torch.device("cpu"))
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=op)
    return float(t.item())


def max_over_ranks(x: float, world: int) -> float:
    """The largest of every rank's value (a time: the job ends with its
    slowest rank)."""
    import torch
    return _reduce_scalar(x, world, torch.distributed.ReduceOp.MAX if world > 1 else None)


def sum_over_ranks(x: float, world: int) -> float:
    import torch
    return _reduce_scalar(x, world, torch.distributed.ReduceOp.SUM if world > 1 else None)


def shard_range(n: int, rank: int, world: int):
    """Rank `rank`'s contiguous share [lo, hi) of n independent items (the
    batched instances shard across GPUs with no exchange)."""
    base, extra = divmod(n, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def bicrystal_run(args, dev, rank=0, world=1):
    """Batched bicrystals: 512 instances of sizes drawn from {64,96,128}^2 x
    {64,96}, undercooling U[0.25, 3] K, anisotropy strength U[0, 1], random
    orientation pairs, stepped together from CUDA-graph replays; outputs
    velocity ratio and grain-boundary inclination per instance."""
    import torch
    from mpf3d.batched import BatchedBicrystals, sample_batch
    # weak scaling: every rank runs its own batch of args.bicrystal_instances
    # instances, drawn from one sample of world * instances
    n_all = args.bicrystal_instances * world
    dims_all, q_all, dT_all, da_all = sample_batch(n_all, seed=SEED)
    lo, hi = shard_range(n_all, rank, world)
    dims, q, dT, da = dims_all[lo:hi], q_all[lo:hi], dT_all[lo:hi], da_all[lo:hi]
    n = hi - lo
    b = BatchedBicrystals(dims, q, dT, da, base_height=16.0, slots=4, device=dev)
    tuned = b.autotune(steps=8) if not args.no_autotune else None
    b.capture(50)
    b.step(50)  # warm-up replay
    torch.cuda.synchronize(dev)
    tuning = b.tuning
    b = BatchedBicrystals(dims, q, dT, da, base_height=16.0, slots=4, device=dev)
    b.tuning = tuning
    b.capture(50)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    res = b.run(args.bicrystal_steps, sample_every=50, graph_steps=50)
    torch.cuda.synchronize(dev)
    wall = max_over_ranks(time.perf_counter() - t0, world)
    cells = sum_over_ranks(b.total_cells, world)
    ratio = res["velocity_ratio"]
    ang = res["gb_angle_deg"]
    fin = np.isfinite(ratio)
    return {"instances": n_all, "steps": args.bicrystal_steps, "cells_per_step": int(cells),
            "wall_s": wall, "cases_per_hour": n_all / wall * 3600.0,
            "cell_steps_per_s": cells * args.bicrystal_steps / wall,
            "velocity_ratio": {"finite": int(fin.sum()),
                               "median": float(np.median(ratio[fin])) if fin.any() else None,
                               "not_finite": {
                                   "front_near_top_before_two_samples": int((res["ratio_status"] == 1).sum()),
                                   "grain2_not_growing": int((res["ratio_status"] == 2).sum()),
                                   "other": int((res["ratio_status"] == 3).sum()),
                                   "instances": [{"dims": list(dims[i]), "undercooling_K": float(dT[i]),
                                                  "delta_a": float(da[i]), "status": int(res["ratio_status"][i])}
                                                 for i in np.flatnonzero(~fin)[:20].tolist()]},
                               "sample_every": 50},
            "gb_inclination_deg": {"finite": int(np.isfinite(ang).sum()),
                                   "median_abs": float(np.nanmedian(np.abs(ang))) if np.isfinite(ang).any()
                                   else None},
            "launches_per_step": 3, "graph_steps": 50,
            "launch_shape": {"work_list_kernels": list(tuned["config"][2:]), "ms_per_step_tuned": tuned["ms_per_step"],
                             "ms_per_step_default": tuned["default_ms_per_step"]} if tuned else None}


def emit(args, rank, world, value, ms, cells, t_e2e, in_bytes, out_bytes, achieved, peak, peak_kind,
         traffic, bytes_per_launch, occ, clk, cpu, final_cnt_sum, extra=None):
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": config_dict(args),
                "e2e": {"value": cells * args.steps * world / t_e2e, "unit": UNIT,
                        "h2d_bytes_per_step": in_bytes / args.steps,
                        "d2h_bytes_per_step": out_bytes / args.steps},
                "gpu_launches": 3 * args.steps,
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak, "traffic": traffic,
                             "peak_source": peak_kind,
                             "bytes_per_cell_step": bytes_per_launch / cells,
                             "bytes_basis": "records of the cells in the tiles each step visits, read + "
                                            "written once (quiet tiles move nothing)",
                             "kernel": f"sweep+general+interface kernels <{args.slots},{2 * args.slots}>",
                             "traffic_unit": "bytes per step (3 launches) over timed steps 1-20, from the "
                                             "committed ncu summary of a 128x128x256 crop scaled 4x by area"},
                "stored_phases_per_cell": {"start": occ[0] / cells, "end": occ[-1] / cells},
                "clocks": clk.summary(),
                "cpu_baseline": cpu}
        line.update(extra or {})
        assert final_cnt_sum == occ[-1], "timed and accounting runs diverged"
        print(json.dumps(line), flush=True)


def run_c3(args):
    """Large single domain in FP32: 1024 x 1024 x 256 cells, 512 grains seeded
    in the bottom 24 layers + liquid (N = 513), started directly in compact
    form from the owner map (the dense field would need 551 GB)."""
    import torch
    from mpf3d import inputs
    from mpf3d.solver import CompactSolver
    dev = torch.device("cuda:0")
    nx, ny, nz, ng, slab = 1024, 1024, 256, 512, 24
    phys = inputs.Physics()
    d = phys.derived()
    t0 = time.perf_counter()
    owner = inputs.voronoi_slab_owner(nx, ny, slab, ng, slab, SEED)
    prof = inputs.tanh_profile(nz, slab, phys.dx, d["delta"])
    temp = inputs.temperature_field(1, 1, nz, phys.T_melt, phys.G, phys.dx, slab)[0, 0]
    q = inputs.random_quaternions(ng, ORIENT_SEED)
    wij, aij, mij = inputs.matrices_for(phys, ng + 1)
    n111 = inputs.rotated_n111(q)
    s = CompactSolver.from_owner(owner, prof, temp, n111, wij, aij, mij, phys, slots=args.slots)
    setup = time.perf_counter() - t0
    s.step(args.warmup)
    tuned = s.autotune(steps=4) if not args.no_autotune else None  # trials restore the state
    torch.cuda.synchronize(dev)
    stream = torch.cuda.current_stream(dev)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clk:
        torch.cuda.synchronize(dev)
        e0.record(stream)
        for i in range(args.steps):
            s.launch_step(args.warmup + i + 1)
        e1.record(stream)
        torch.cuda.synchronize(dev)
    s.check()
    ms = e0.elapsed_time(e1)
    cells = nx * ny * nz
    line = {"metric": "3D cell-steps/s (FP32 compact step, 1024x1024x256, N=513)",
            "value": cells * args.steps / (ms / 1e3), "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": "1024x1024x256, 512 grains in the bottom 24 layers + liquid (N=513), "
                                   "anisotropy+torque, uniform cooling, FP32 compact, started from the owner map",
                       "slots": s.slots, "state_bytes_per_buffer": s.state_bytes()},
            "setup_s": setup, "stored_phases_per_cell_end": float(s.stored_counts().double().mean().item()),
            "clocks": clk.summary(), "gpu_launches": 3 * args.steps,
            "launch_shape": {"config": list(tuned["config"]), "sweep_tma": bool(s.sweep_tma),
                             "ms_per_step_tuned": tuned["ms_per_step"],
                             "ms_per_step_default": tuned["default_ms_per_step"]} if tuned else None}
    print(json.dumps(line), flush=True)


def run_accuracy_study(args):
    """The FP32-vs-FP64 divergence study of the bench workload (or of the
    grid, grains and slab given) over --steps steps (the default bench line
    runs only the first 100)."""
    import torch
    from mpf3d import inputs
    dev = torch.device("cuda:0")
    phys = inputs.Physics()
    d = phys.derived()
    nx, ny, nz = GRID
    owner = torch.from_numpy(workload_owner(nx, ny, nz)).to(dev)
    prof = torch.from_numpy(inputs.tanh_profile(nz, SLAB, phys.dx, d["delta"])).to(dev)
    temp = inputs.temperature_field(1, 1, nz, phys.T_melt, phys.G, phys.dx, SLAB)[0, 0]
    n111, wij, aij, mij = workload_inputs(phys)
    phi0 = dense_phi_on_device(owner, prof, torch)
    args.accuracy_steps = args.steps
    print(json.dumps({"workload": "accuracy study", **accuracy_run(args, phi0, temp, n111, wij, aij, mij, phys,
                                                                     dev)}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c2", choices=["c2", "c3", "accuracy", "c5"],
                    help="c2: the 256^3 bench line; c3: the 1024x1024x256 large-domain run")
    ap.add_argument("--slots", type=int, default=16)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end run (profiling)")
    ap.add_argument("--no-autotune", action="store_true", help="use the default launch shape")
    ap.add_argument("--no-graph", action="store_true", help="launch the timed steps eagerly, not from a CUDA graph")
    ap.add_argument("--no-gemm", action="store_true", help="skip the surrogate GEMM measurement")
    ap.add_argument("--no-dense-reference", action="store_true",
                    help="skip timing the reference-numerics dense kernels on the same workload")
    ap.add_argument("--grid", type=int, nargs=3, default=None,
                    help="override the 256^3 grid (smaller cases for profiling)")
    ap.add_argument("--accuracy-steps", type=int, default=100)
    ap.add_argument("--no-accuracy", action="store_true")
    ap.add_argument("--bicrystal-steps", type=int, default=3000)
    ap.add_argument("--bicrystal-instances", type=int, default=512)
    ap.add_argument("--no-bicrystal", action="store_true")
    ap.add_argument("--candidates", type=int, default=65536)
    ap.add_argument("--exhaustive", action="store_true", help="c5: also simulate every candidate")
    ap.add_argument("--screen-rounds", type=int, default=2, help="c5: surrogate refit rounds")
    ap.add_argument("--recheck", type=int, default=1024, help="c5: candidates re-simulated per refit round")
    ap.add_argument("--c5-config", action="store_true",
                    help="c5: instances of {64,96,128}^2 x {64,96} cells stepped 3000 steps (the stated "
                         "configuration) instead of 32x32x64 for 300 steps")
    ap.add_argument("--slab", type=int, default=None,
                    help="height of the solid Voronoi slab and of the initial front (default 32; the "
                         "1024x1024x256 workload uses 24)")
    ap.add_argument("--grains", type=int, default=None,
                    help="grains of the Voronoi slab (default 64; a crop of the 256^3 workload keeps the grain "
                         "density with 64 * nx * ny / 256^2)")
    args = ap.parse_args()
    global GRID, N_GRAINS, SLAB
    if args.grid:
        GRID = tuple(args.grid)
    if args.grains:
        N_GRAINS = int(args.grains)
    if args.slab:
        SLAB = int(args.slab)
    if args.warmup < 3:
        args.warmup = 3
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1 and args.impl == "ours":
        import torch
        torch.distributed.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    if args.impl == "reference":
        run_reference(args, rank)
    elif args.workload == "c3":
        run_c3(args)
    elif args.workload == "accuracy":
        run_accuracy_study(args)
    elif args.workload == "c5":
        from mpf3d.screen import screen
        if args.c5_config:
            # the stated configuration: instances of the batched-bicrystal
            # workload's sizes ({64,96,128}^2 x {64,96}), 3000 steps each
            rep = screen(n_candidates=args.candidates, exhaustive=args.exhaustive, seed=SEED,
                         rounds=args.screen_rounds, recheck=args.recheck, dims="ragged", steps=3000,
                         batch=512, sample_every=50)
        else:
            rep = screen(n_candidates=args.candidates, exhaustive=args.exhaustive, seed=SEED,
                         rounds=args.screen_rounds, recheck=args.recheck)
        print(json.dumps({"workload": "surrogate-screened orientation scan", **rep}), flush=True)
    else:
        run_ours(args, rank, world)
    if world > 1 and args.impl == "ours":
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
