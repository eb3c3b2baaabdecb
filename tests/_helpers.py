"""Shared helpers of the test suite."""
import glob
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")


def golden_files(kind="run"):
    """Golden fixtures of one kind: "run" (3D step sequences), "run2d" (2D
    step sequences) or "apt" (APT known answers)."""
    out = []
    for f in sorted(glob.glob(os.path.join(GOLDEN, "*.npz"))):
        g = np.load(f)
        if "phi0" not in g.files:
            continue  # analysis fixtures (groove_metrics.npz)
        if "phi" not in g.files:
            k = "apt"
        else:
            k = "run2d" if g["phi0"].ndim == 3 else "run"
        if k == kind:
            out.append(f)
    return out


def golden_id(f):
    return os.path.basename(f)[:-4]


def valid_mf_equal(mf_a, mf_b, nf):
    """mf entries below nf agree (rows at or above nf are stale by design)."""
    d = min(mf_a.shape[0], mf_b.shape[0])
    depth = np.arange(d).reshape((d,) + (1,) * nf.ndim)
    mask = depth < nf[None]
    if int(nf.max()) > d:
        return False
    return bool(np.array_equal(np.where(mask, mf_a[:d], -1), np.where(mask, mf_b[:d], -1)))
