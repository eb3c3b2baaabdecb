"""Autotuner for the compact step's launch shape.

The reference launches every kernel with a fixed [4, 4, 4] block
(config_3d.yaml gpu.threads_per_block).  Here the shape -- cells per sweep
thread along z, sweep block height, the grid and block sizes of the two
work-list kernels, and whether the sweep stages its heads in shared memory by
TMA -- is searched per problem (grid, phases, slots, model
switches, GPU) by timing each candidate on the solver's own state with CUDA
events, restoring the state before every trial.  All shapes compute identical
results.  Winners are cached in a JSON file (MPF3D_TUNING_CACHE, default
~/.cache/mpf3d/tuning.json).
"""

from __future__ import annotations

import itertools
import json
import os

from . import _lib

DEFAULT = (4, 8, 8, 256, 8, 128)
SWEEP = [(zb, by) for zb in (2, 4, 8) for by in (4, 8, 16)]
QUEUE = [(g, gt, i, it) for (g, gt), (i, it) in itertools.product([(4, 256), (8, 256), (16, 128), (32, 128)],
                                                                   [(4, 128), (8, 128), (16, 64), (32, 64)])]


def cache_path() -> str:
    return os.path.abspath(os.environ.get("MPF3D_TUNING_CACHE",
                                          os.path.join(os.path.expanduser("~"), ".cache", "mpf3d", "tuning.json")))


def make(cfg) -> _lib.Tuning:
    t = _lib.Tuning()
    (t.sweep_zb, t.sweep_by, t.general_blocks_per_sm, t.general_threads, t.iface_blocks_per_sm,
     t.iface_threads) = (int(v) for v in cfg)
    return t


def key_of(solver) -> str:
    import torch

    name = torch.cuda.get_device_name(solver.device)
    return (f"{name}|{solver.nx}x{solver.ny}x{solver.nz}|N{solver.N}|S{solver.slots}|"
            f"a{int(solver.anisotropy)}t{int(solver.torque)}")


def _load() -> dict:
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(db: dict) -> None:
    p = cache_path()
    os.makedirs(os.path.dirname(p), exist_ok=True)
    tmp = p + f".tmp{os.getpid()}"
    with open(tmp, "w") as f:
        json.dump(db, f, indent=1, sort_keys=True)
    os.replace(tmp, p)


def time_config(solver, cfg, steps: int, sweep_tma: bool = False) -> float:
    """Milliseconds per step of `cfg` (and the sweep form) on the solver's
    current state (restored afterwards)."""
    import torch

    snap = [t.clone() for t in solver.buf[solver.cur]]
    cur, count = solver.cur, solver.step_count
    prev, prev_tma = solver.tuning, solver.sweep_tma
    solver.tuning = make(cfg)
    solver.sweep_tma = sweep_tma
    solver.forget_history()  # the trial starts from the snapshot, not from the last step
    stream = torch.cuda.current_stream(solver.device)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    try:
        solver.launch_step(count + 1)  # warm-up of this shape
        e0.record(stream)
        for i in range(steps):
            solver.launch_step(count + 2 + i)
        e1.record(stream)
        torch.cuda.synchronize(solver.device)
        ms = e0.elapsed_time(e1) / steps
    finally:
        solver.tuning, solver.sweep_tma = prev, prev_tma
        solver.cur, solver.step_count = cur, count
        for dst, src in zip(solver.buf[cur], snap):
            dst.copy_(src)
        solver.forget_history()
    return ms


def tune(solver, steps: int = 8, use_cache: bool = True) -> dict:
    """Search the launch shape for `solver`; returns {"config", "ms_per_step",
    "default_ms_per_step", "trials"} and sets solver.tuning."""
    key = key_of(solver)
    db = _load() if use_cache else {}
    if use_cache and key in db:
        solver.tuning = make(db[key]["config"])
        solver.sweep_tma = bool(db[key].get("sweep_tma", False))
        return db[key]
    trials = {}
    base = time_config(solver, DEFAULT, steps)
    trials[str(DEFAULT)] = base
    best, best_ms = DEFAULT, base
    # stage 1: the sweep shape with the default work-list shape
    for zb, by in SWEEP:
        cfg = (zb, by) + DEFAULT[2:]
        if str(cfg) not in trials:
            trials[str(cfg)] = time_config(solver, cfg, steps)
        if trials[str(cfg)] < best_ms:
            best, best_ms = cfg, trials[str(cfg)]
    # stage 2: the work-list kernels with the best sweep shape
    for q in QUEUE:
        cfg = best[:2] + q
        if str(cfg) not in trials:
            trials[str(cfg)] = time_config(solver, cfg, steps)
        if trials[str(cfg)] < best_ms:
            best, best_ms = cfg, trials[str(cfg)]
    # stage 3: the sweep with its heads staged in shared memory by TMA
    tma = False
    if solver.nx % 4 == 0:
        ms = time_config(solver, best, steps, sweep_tma=True)
        trials[str(best) + " tma"] = ms
        if ms < best_ms:
            tma, best_ms = True, ms
    solver.tuning = make(best)
    solver.sweep_tma = tma
    rec = {"config": list(best), "sweep_tma": tma, "ms_per_step": best_ms, "default_ms_per_step": base,
           "trials": trials}
    if use_cache:
        db[key] = rec
        _store(db)
    return rec


def tune_batched(batch, steps: int = 8, use_cache: bool = True) -> dict:
    """Search the grid and block sizes of the batched step's two work-list
    kernels (the QUEUE candidates) on the batch's own state, restored after
    every trial; sets batch.tuning.  Cached per (GPU, instance count, total
    cells, slots, model switches)."""
    import torch

    name = torch.cuda.get_device_name(batch.device)
    key = (f"batched|{name}|n{batch.n}|cells{batch.total_cells}|S{batch.slots}|"
           f"a{int(batch.anisotropy)}t{int(batch.torque)}")
    db = _load() if use_cache else {}
    if use_cache and key in db:
        batch.tuning = make(db[key]["config"])
        return db[key]
    if batch.graph is not None:
        raise RuntimeError("tune the batch before capturing a graph of its steps")

    def trial(cfg):
        snap = [t.clone() for t in batch.buf[batch.cur]]
        cur, count = batch.cur, batch.step_count
        prev = batch.tuning
        batch.tuning = make(cfg)
        stream = torch.cuda.current_stream(batch.device)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        try:
            batch.launch_step()
            e0.record(stream)
            for _ in range(steps):
                batch.launch_step()
            e1.record(stream)
            torch.cuda.synchronize(batch.device)
            return e0.elapsed_time(e1) / steps
        finally:
            batch.tuning = prev
            batch.cur, batch.step_count = cur, count
            for dst, src in zip(batch.buf[cur], snap):
                dst.copy_(src)
            batch.forget_history()

    trials = {}
    base = trial(DEFAULT)
    trials[str(DEFAULT)] = base
    best, best_ms = DEFAULT, base
    for q in QUEUE:
        cfg = DEFAULT[:2] + q
        if str(cfg) not in trials:
            trials[str(cfg)] = trial(cfg)
        if trials[str(cfg)] < best_ms:
            best, best_ms = cfg, trials[str(cfg)]
    batch.tuning = make(best)
    rec = {"config": list(best), "ms_per_step": best_ms, "default_ms_per_step": base, "trials": trials}
    if use_cache:
        db[key] = rec
        _store(db)
    return rec
