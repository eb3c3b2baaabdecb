"""Surrogate-screened orientation scan.

A batch of candidate grain pairs (two orientations, undercooling, anisotropy
strength) is ranked by the surrogate; the plain FP32 batched solver then
re-simulates the top-k plus a random audit sample, which both checks the
ranking and serves as the fallback answer.  The reference's counterpart is the
serial scan of run_orientation_scan_3d.py:686-841, which simulates every
candidate.
"""

from __future__ import annotations

import time

import numpy as np

from .batched import BatchedBicrystals
from .surrogate import Surrogate


def bounded(y: np.ndarray) -> np.ndarray:
    """Training form of the targets: the velocity ratio r mapped to
    (r - 1)/(|r| + 1) -- (v1 - v2)/(v1 + v2) for growing grains, bounded and
    monotone in r -- and the inclination in units of 45 degrees."""
    y = np.asarray(y, np.float64)
    return np.stack([(y[:, 0] - 1.0) / (np.abs(y[:, 0]) + 1.0), y[:, 1] / 45.0], 1)


def best_simulated(known: dict, k: int) -> np.ndarray:
    """The k candidates with the largest simulated value among `known`
    (candidate -> value; NaN ranks last)."""
    ids = np.fromiter(known.keys(), dtype=np.int64, count=len(known))
    vals = np.fromiter(known.values(), dtype=np.float64, count=len(known))
    return ids[np.argsort(-np.where(np.isfinite(vals), vals, -np.inf), kind="stable")[:k]]


def sample_pairs(n: int, seed: int, dT_range=(0.25, 3.0), delta_a_range=(0.0, 1.0)):
    rng = np.random.default_rng(seed)
    q = rng.standard_normal((n, 2, 4))
    q /= np.linalg.norm(q, axis=2, keepdims=True)
    return q[:, 0], q[:, 1], rng.uniform(*dT_range, n), rng.uniform(*delta_a_range, n)


def candidate_dims(n: int, seed: int, sizes_xy=(64, 96, 128), sizes_z=(64, 96)):
    """Per-candidate grid sizes drawn uniformly from sizes_xy^2 x sizes_z (the
    batched-bicrystal workload's instance sizes)."""
    rng = np.random.default_rng(seed)
    return [(int(rng.choice(sizes_xy)), int(rng.choice(sizes_xy)), int(rng.choice(sizes_z))) for _ in range(n)]


def simulate(q1, q2, dT, da, dims=(32, 32, 64), steps=300, sample_every=10, batch=4096, base_height=16.0,
             device="cuda:0"):
    """Velocity ratio and grain-boundary inclination of every pair, simulated
    in batches of `batch` instances; dims is one (nx, ny, nz) for every pair or
    a list with one per pair.  Returns ([n, 2] targets, GPU seconds)."""
    import torch

    n = len(q1)
    per_pair = isinstance(dims, list)
    out = np.full((n, 2), np.nan)
    t0 = time.perf_counter()
    for s in range(0, n, batch):
        e = min(n, s + batch)
        q = np.stack([q1[s:e], q2[s:e]], 1)
        b = BatchedBicrystals(dims[s:e] if per_pair else [dims] * (e - s), q, dT[s:e], da[s:e],
                              base_height=base_height, slots=4, device=device)
        b.capture(sample_every if sample_every % 2 == 0 else 2 * sample_every)
        r = b.run(steps, sample_every=sample_every, graph_steps=0)
        out[s:e, 0] = r["velocity_ratio"]
        out[s:e, 1] = r["gb_angle_deg"]
        del b
    torch.cuda.synchronize()
    return out, time.perf_counter() - t0


def screen(n_candidates=65536, n_train=512, top_k=256, n_audit=256, seed=0, dims=(32, 32, 64), steps=300,
           epochs=300, objective=0, exhaustive=False, rounds=1, recheck=1024, device="cuda:0", batch=4096,
           sample_every=10):
    """Rank n_candidates pairs by the surrogate's prediction of target
    `objective` (0 velocity ratio, 1 grain-boundary inclination; larger is
    better) and check it by re-simulation.  Errors and objective values are
    reported in the bounded training form (see `bounded`).

    rounds > 1 adds refinement rounds: a surrogate is refitted on every
    candidate simulated so far (the random training set, the checked top and
    the audit sample), and its top `recheck` candidates that have not been
    simulated yet are simulated.  The answer (`final`) is then the top_k of
    all simulated candidates by their simulated value.  Every GPU second of
    the refinement counts in `screened_total`.  dims is one grid for every
    candidate, or "ragged": per-candidate sizes from candidate_dims (the
    batched-bicrystal workload's {64,96,128}^2 x {64,96}).  Returns a report
    dict."""
    import torch

    q1, q2, dT, da = sample_pairs(n_candidates, seed)
    dims_all = candidate_dims(n_candidates, seed + 7) if dims == "ragged" else None

    def dims_of(idx):
        return [dims_all[i] for i in np.asarray(idx).tolist()] if dims_all is not None else dims

    def sim(idx):
        return simulate(q1[idx], q2[idx], dT[idx], da[idx], dims_of(idx), steps, sample_every=sample_every,
                        batch=batch, device=device)

    rng = np.random.default_rng(seed + 1)
    train_idx = rng.choice(n_candidates, n_train, replace=False)
    y_train, t_train = sim(train_idx)
    t0 = time.perf_counter()
    s = Surrogate(seed=seed, device=device)
    hist = s.fit(q1[train_idx], q2[train_idx], dT[train_idx], da[train_idx], bounded(y_train), epochs=epochs,
                 batch=128, lr=2e-3)
    torch.cuda.synchronize()
    t_fit = time.perf_counter() - t0
    t0 = time.perf_counter()
    pred = s.predict(q1, q2, dT, da)
    torch.cuda.synchronize()
    t_pred = time.perf_counter() - t0
    order = np.argsort(-pred[:, objective])
    top = order[:top_k]
    audit = rng.choice(n_candidates, n_audit, replace=False)
    chk_idx = np.concatenate([top, audit])
    y_chk, t_chk = sim(chk_idx)
    y_chk = bounded(y_chk)
    p_chk = pred[chk_idx]

    def err(a, b):
        ok = np.all(np.isfinite(a), 1) & np.all(np.isfinite(b), 1)
        d = a[ok] - b[ok]
        corr = [float(np.corrcoef(a[ok, c], b[ok, c])[0, 1]) if ok.sum() > 2 else float("nan") for c in range(2)]
        return {"rmse": np.sqrt((d ** 2).mean(0)).tolist(), "corr": corr, "n": int(ok.sum())}

    y_top, y_aud = y_chk[:top_k, objective], y_chk[top_k:, objective]
    report = {
        "candidates": n_candidates, "train": n_train, "top_k": top_k, "audit": n_audit,
        "dims": dims if isinstance(dims, str) else list(dims), "steps": steps, "objective": ["velocity_ratio", "gb_inclination_deg"][objective],
        "train_loss_first_last": [hist[0], hist[-1]],
        "surrogate_error_top": err(p_chk[:top_k], y_chk[:top_k]),
        "surrogate_error_audit": err(p_chk[top_k:], y_chk[top_k:]),
        "objective_mean_top_simulated": float(np.nanmean(y_top)),
        "objective_mean_random_simulated": float(np.nanmean(y_aud)),
        "gain_over_random_same_budget": float(np.nanmean(y_top) - np.nanmean(y_aud)),
        "gpu_seconds": {"train_sims": t_train, "fit": t_fit, "predict": t_pred, "recheck_sims": t_chk},
    }
    known = {}  # candidate -> simulated objective (bounded form)
    for i, v in zip(train_idx.tolist(), bounded(y_train)[:, objective].tolist()):
        known[i] = v
    for i, v in zip(chk_idx.tolist(), y_chk[:, objective].tolist()):
        known[i] = v
    t_refine = 0.0
    for r in range(1, rounds):
        t0 = time.perf_counter()
        idx = np.fromiter(known.keys(), dtype=np.int64)
        yk = np.full((len(idx), 2), np.nan)
        yk[:, objective] = np.fromiter(known.values(), dtype=np.float64)
        yk[:, 1 - objective] = 0.0  # only the objective is refitted
        s_r = Surrogate(seed=seed + r, device=device)
        s_r.fit(q1[idx], q2[idx], dT[idx], da[idx], yk, epochs=epochs, batch=512, lr=2e-3,
                weights=(1.0, 0.0) if objective == 0 else (0.0, 1.0))
        pred_r = s_r.predict(q1, q2, dT, da)
        torch.cuda.synchronize()
        new = [i for i in np.argsort(-pred_r[:, objective])[:recheck].tolist() if i not in known]
        t_refine += time.perf_counter() - t0
        if new:
            new = np.array(new)
            y_new, t_new = sim(new)
            t_refine += t_new
            for i, v in zip(new.tolist(), bounded(y_new)[:, objective].tolist()):
                known[i] = v
    final_top = best_simulated(known, top_k)
    report["final"] = {"rounds": rounds, "recheck": recheck if rounds > 1 else 0, "simulated": len(known),
                       "objective_mean": float(np.nanmean([known[i] for i in final_top.tolist()]))}
    report["gpu_seconds"]["refine"] = t_refine
    screened = t_train + t_fit + t_pred + t_chk + t_refine
    report["gpu_seconds"]["screened_total"] = screened
    if exhaustive:
        y_all, t_all = sim(np.arange(n_candidates))
        y_all = bounded(y_all)
        truth = y_all[:, objective]
        fin = np.isfinite(truth)
        true_top = np.argsort(-np.where(fin, truth, -np.inf))[:top_k]
        report["exhaustive"] = {
            "gpu_seconds": t_all, "speedup_vs_exhaustive": t_all / screened,
            "top_k_overlap": len(set(top.tolist()) & set(true_top.tolist())) / top_k,
            "final_top_k_overlap": len(set(final_top.tolist()) & set(true_top.tolist())) / top_k,
            "final_top_true_mean": float(np.nanmean(truth[final_top])),
            "true_top_mean": float(np.nanmean(truth[true_top])),
            "surrogate_top_true_mean": float(np.nanmean(truth[top])),
            "surrogate_error_all": err(pred, y_all),
        }
    return report
