"""Orientation surrogate: a 4-layer MLP (10 -> 256 -> 256 -> 256 -> 2, SiLU)
trained on the batched bicrystal engine's outputs.  It maps a grain pair's
orientations, the undercooling and the anisotropy strength to the growth
velocity ratio and the grain-boundary inclination.

Weights are stored in FP32 (Adam master copy) and BF16 (the copy the
tensor-core GEMMs read); every matrix product runs in libmpf3d's
`mpf3d_gemm_bf16` on the fifth-generation tensor cores (tcgen05, FP32
accumulate in tensor memory): the forward products X W^T on the TMA-fed
pipelined kernel, the gradients dZ W and dZ^T X on the kernel that gathers
transposed operands into shared memory.  The activation derivative, loss and
Adam run in its elementwise kernels.  Torch provides device memory only.

No reference counterpart: the reference has no learned component; it scans
orientations one simulation at a time (run_orientation_scan_3d.py:686-841).
"""

from __future__ import annotations

import ctypes

import numpy as np

from . import _lib

IN_FEATURES = 10     # physical inputs: 2 quaternions, undercooling, anisotropy strength
DERIVED = 4          # fixed facet-alignment features computed from the quaternions
K1 = 16  # input columns of the first GEMM (k granularity of the tensor-core tile)
HIDDEN = 256
OUT = 2
LAYERS = [(K1, HIDDEN, 1), (HIDDEN, HIDDEN, 1), (HIDDEN, HIDDEN, 1), (HIDDEN, OUT, 0)]  # (K, N, act)


def n_params(derived: bool = False) -> int:
    """Trainable parameters of the 10 -> 256 -> 256 -> 256 -> 2 network (with
    `derived`, also the first-layer weights of the 4 derived features)."""
    k = IN_FEATURES + (DERIVED if derived else 0)
    return k * HIDDEN + HIDDEN + 2 * (HIDDEN * HIDDEN + HIDDEN) + HIDDEN * OUT + OUT


def canonical(q: np.ndarray) -> np.ndarray:
    """Quaternions (x, y, z, w) on the w >= 0 hemisphere (q and -q are the
    same rotation)."""
    q = np.asarray(q, np.float64)
    return np.where(q[..., 3:4] < 0, -q, q)


def cubic_group() -> np.ndarray:
    """The 24 proper rotations of the cube as (x, y, z, w) quaternions; the
    {111} normal set, and so the physics, is invariant under them."""
    s = 0.5 ** 0.5
    qs = [(0, 0, 0, 1), (1, 0, 0, 0), (0, 1, 0, 0), (0, 0, 1, 0)]
    for ax in np.eye(3):
        for sign in (1, -1):
            qs.append(tuple(sign * s * ax) + (s,))
    for a, b in ((0, 1), (0, 2), (1, 2)):
        for sign in (1, -1):
            v = np.zeros(3)
            v[a], v[b] = s, sign * s
            qs.append(tuple(v) + (0.0,))
    for sx in (1, -1):
        for sy in (1, -1):
            for sz in (1, -1):
                if sx * sy * sz > 0:
                    qs.append((0.5 * sx, 0.5 * sy, 0.5 * sz, 0.5))
                    qs.append((-0.5 * sx, -0.5 * sy, -0.5 * sz, 0.5))
    out = np.array(qs, np.float64)
    assert out.shape == (24, 4)
    return out


def qmul(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Hamilton product of (x, y, z, w) quaternions (broadcasting)."""
    ax, ay, az, aw = np.moveaxis(a, -1, 0)
    bx, by, bz, bw = np.moveaxis(b, -1, 0)
    return np.stack([aw * bx + ax * bw + ay * bz - az * by,
                     aw * by - ax * bz + ay * bw + az * bx,
                     aw * bz + ax * by - ay * bx + az * bw,
                     aw * bw - ax * bx - ay * by - az * bz], -1)


def facet_alignment(q: np.ndarray) -> np.ndarray:
    """[M, 2]: the two largest |n . z| over a grain's rotated {111} normals --
    how close its nearest facets lie to the growth direction z, which sets
    a(theta) and b(theta) of a front normal to z.  Invariant under the cubic
    group and under q -> -q."""
    q = np.asarray(q, np.float64)
    x, y, z, w = np.moveaxis(q / np.linalg.norm(q, axis=-1, keepdims=True), -1, 0)
    # third row of the rotation matrix: z components of the rotated axes
    r = np.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], -1)
    base = np.array([[1, 1, 1], [1, 1, -1], [1, -1, 1], [-1, 1, 1]], np.float64) / np.sqrt(3.0)
    c = np.sort(np.abs(r @ base.T), axis=-1)
    return c[..., ::-1][..., :2]


def features(q1, q2, undercooling, delta_a, dT_range=(0.25, 3.0)) -> np.ndarray:
    """[M, 14] network input: the 10 physical inputs -- both canonical
    quaternions, undercooling and anisotropy strength mapped to [-1, 1] --
    followed by 4 fixed invariant features of the quaternions (the facet
    alignment of each grain with z), which occupy 4 of the 6 padding columns
    of the first GEMM."""
    q1 = canonical(q1)
    q2 = canonical(q2)
    lo, hi = dT_range
    dT = (np.asarray(undercooling, np.float64) - lo) / (hi - lo) * 2.0 - 1.0
    da = np.asarray(delta_a, np.float64) * 2.0 - 1.0
    f1 = facet_alignment(q1) * 2.0 - 1.0
    f2 = facet_alignment(q2) * 2.0 - 1.0
    return np.concatenate([q1, q2, dT[:, None], da[:, None], f1, f2], 1).astype(np.float32)


def augment(q1, q2, rng) -> tuple:
    """Apply an independent random cubic symmetry to each grain's orientation
    (right multiplication: a rotation of the crystal frame)."""
    G = cubic_group()
    a = G[rng.integers(0, 24, len(q1))]
    b = G[rng.integers(0, 24, len(q2))]
    return qmul(q1, a), qmul(q2, b)


class Surrogate:
    def __init__(self, seed: int = 0, device="cuda:0"):
        import torch

        self.torch = torch
        self.device = torch.device(device)
        rng = np.random.default_rng(seed)
        self.offsets = []
        chunks = []
        off = 0
        for K, N, _ in LAYERS:
            fan_in = IN_FEATURES if K == K1 else K
            bound = 1.0 / np.sqrt(fan_in)
            W = rng.uniform(-bound, bound, (N, K)).astype(np.float32)
            if K == K1:
                W[:, IN_FEATURES + DERIVED:] = 0.0
            b = rng.uniform(-bound, bound, N).astype(np.float32)
            self.offsets.append((off, off + N * K))
            chunks += [W.ravel(), b]
            off += N * K + N
        self.size = off
        t = torch
        self.w = t.from_numpy(np.concatenate(chunks)).to(self.device)
        self.w16 = t.empty(self.size, dtype=t.int16, device=self.device)
        self.g = t.zeros(self.size, dtype=t.float32, device=self.device)
        self.m = t.zeros_like(self.w)
        self.v = t.zeros_like(self.w)
        self.adam_step = 0
        self._bf16(self.w, self.w16)
        self.mean = np.zeros(OUT, np.float32)
        self.std = np.ones(OUT, np.float32)
        self.loss_w = t.ones(OUT, dtype=t.float32, device=self.device)
        # device error word of the tcgen05 GEMM (MPF3D_DEV_GEMM_ABORT), read by check()
        self.gemm_err = t.zeros(1, dtype=t.int32, device=self.device)

    # -- helpers -------------------------------------------------------------------
    def _s(self):
        return self.torch.cuda.current_stream(self.device).cuda_stream or None

    def _bf16(self, x, y):
        _lib.check(_lib.lib().mpf3d_f32_to_bf16(x.data_ptr(), y.data_ptr(), x.numel(), self._s()), "f32_to_bf16")

    def _W(self, layer, bf16=True):
        o, ob = self.offsets[layer]
        K, N, _ = LAYERS[layer]
        buf = self.w16 if bf16 else self.w
        return buf.narrow(0, o, N * K), self.w.narrow(0, ob, N)

    def _gemm(self, M, N, K, A, sam, sak, B, sbk, sbn, bias, act, Z, Y, ldy, y_bf16, beta=0):
        rc = _lib.lib().mpf3d_gemm_bf16(M, N, K, A.data_ptr(), sam, sak, B.data_ptr(), sbk, sbn,
                                        bias.data_ptr() if bias is not None else None, act,
                                        Z.data_ptr() if Z is not None else None, Y.data_ptr(), ldy, int(y_bf16),
                                        beta, self.gemm_err.data_ptr(), self._s())
        _lib.check(rc, "gemm_bf16")

    def prepare(self, X: np.ndarray):
        """[M, <=16] float features -> zero-padded BF16 device input [M, 16]."""
        t = self.torch
        M = X.shape[0]
        xp = np.zeros((M, K1), np.float32)
        xp[:, :X.shape[1]] = X
        x32 = t.from_numpy(xp).to(self.device)
        x16 = t.empty((M, K1), dtype=t.int16, device=self.device)
        self._bf16(x32, x16)
        return x16

    # -- network -------------------------------------------------------------------
    def forward(self, x16, keep: bool = False):
        """Raw (standardised) outputs [M, 2] FP32; keep=True stores what the
        backward pass needs."""
        t = self.torch
        M = x16.shape[0]
        h = x16
        saved = [x16]
        for layer, (K, N, act) in enumerate(LAYERS):
            W16, b = self._W(layer)
            last = layer == len(LAYERS) - 1
            Z = t.empty((M, N), dtype=t.float32, device=self.device) if (keep and act) else None
            Y = t.empty((M, N), dtype=t.float32 if last else t.int16, device=self.device)
            self._gemm(M, N, K, h, K, 1, W16, 1, K, b, act, Z, Y, N, not last)
            saved.append((Z, Y))
            h = Y
        if keep:
            self._saved = saved
        return h

    def backward(self, dout) -> None:
        """Gradients of the loss w.r.t. all parameters into self.g, given the
        FP32 gradient w.r.t. the outputs [M, 2]."""
        t = self.torch
        L = _lib.lib()
        saved = self._saved
        M = dout.shape[0]
        dY = dout
        for layer in range(len(LAYERS) - 1, -1, -1):
            K, N, act = LAYERS[layer]
            Z, _ = saved[layer + 1]
            Hin = saved[layer] if layer == 0 else saved[layer][1]
            dZ16 = t.empty((M, N), dtype=t.int16, device=self.device)
            dZ32 = t.empty((M, N), dtype=t.float32, device=self.device)
            _lib.check(L.mpf3d_act_backward(dY.data_ptr(), Z.data_ptr() if Z is not None else None, act, M * N,
                                            dZ16.data_ptr(), dZ32.data_ptr(), self._s()), "act_backward")
            o, ob = self.offsets[layer]
            gW = self.g.narrow(0, o, N * K)
            gb = self.g.narrow(0, ob, N)
            # dW[n][k] = sum_m dZ[m][n] Hin[m][k]
            self._gemm(N, K, M, dZ16, 1, N, Hin, K, 1, None, 0, None, gW, K, False)
            _lib.check(L.mpf3d_colsum(dZ32.data_ptr(), M, N, N, gb.data_ptr(), self._s()), "colsum")
            if layer > 0:
                W16, _ = self._W(layer)
                dH = t.empty((M, K), dtype=t.float32, device=self.device)
                # dH[m][k] = sum_n dZ[m][n] W[n][k]
                self._gemm(M, K, N, dZ16, N, 1, W16, K, 1, None, 0, None, dH, K, False)
                dY = dH
        # the padded input columns carry no parameters
        o, _ = self.offsets[0]
        self.g.narrow(0, o, HIDDEN * K1).view(HIDDEN, K1)[:, IN_FEATURES + DERIVED:] = 0.0

    def loss_and_grad(self, x16, target):
        """Weighted MSE on standardised targets; fills self.g, returns the loss."""
        t = self.torch
        M = x16.shape[0]
        out = self.forward(x16, keep=True)
        dout = t.empty_like(out)
        loss = t.zeros(1, dtype=t.float32, device=self.device)
        _lib.check(_lib.lib().mpf3d_mse(out.data_ptr(), OUT, target.data_ptr(), M, OUT, self.loss_w.data_ptr(),
                                        dout.data_ptr(), loss.data_ptr(), self._s()), "mse")
        self.backward(dout)
        return loss

    def adam(self, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8, weight_decay=0.0) -> None:
        self.adam_step += 1
        _lib.check(_lib.lib().mpf3d_adam(self.w.data_ptr(), self.m.data_ptr(), self.v.data_ptr(), self.g.data_ptr(),
                                         self.w16.data_ptr(), self.size, lr, b1, b2, eps, self.adam_step,
                                         weight_decay, self._s()), "adam")

    # -- user API ------------------------------------------------------------------
    def fit(self, q1, q2, undercooling, delta_a, targets, epochs=400, batch=512, lr=2e-3, seed=0,
            augment_symmetry=True, weights=(1.0, 1.0)):
        """Train on (orientation pair, undercooling, anisotropy) -> targets [M, 2]
        (NaN rows dropped); returns the loss history."""
        t = self.torch
        targets = np.asarray(targets, np.float64)
        ok = np.all(np.isfinite(targets), 1)
        q1, q2 = np.asarray(q1)[ok], np.asarray(q2)[ok]
        dT, da, Y = np.asarray(undercooling)[ok], np.asarray(delta_a)[ok], targets[ok]
        self.mean = Y.mean(0).astype(np.float32)
        self.std = np.maximum(Y.std(0), 1e-6).astype(np.float32)
        Ys = t.from_numpy(((Y - self.mean) / self.std).astype(np.float32)).to(self.device)
        self.loss_w = t.tensor(weights, dtype=t.float32, device=self.device)
        rng = np.random.default_rng(seed)
        n = len(Y)
        hist = []
        for ep in range(epochs):
            perm = rng.permutation(n)
            a1, a2 = augment(q1, q2, rng) if augment_symmetry else (q1, q2)
            X = features(a1, a2, dT, da)
            x16 = self.prepare(X)
            ep_loss = 0.0
            for s in range(0, n, batch):
                idx = t.from_numpy(perm[s:s + batch]).to(self.device)
                xb = x16.index_select(0, idx).contiguous()
                yb = Ys.index_select(0, idx).contiguous()
                loss = self.loss_and_grad(xb, yb)
                self.adam(lr=lr * (0.5 * (1 + np.cos(np.pi * ep / epochs))))
                ep_loss += float(loss.item()) * len(idx) / n
            hist.append(ep_loss)
        self.check()
        return hist

    def check(self) -> None:
        """Raise if a tcgen05 GEMM of this network aborted on a wait that ran out."""
        v = int(self.gemm_err.item())
        if v:
            self.gemm_err.zero_()
            raise RuntimeError("surrogate GEMM device error: " + _lib.describe_dev_error(v))

    def predict(self, q1, q2, undercooling, delta_a, chunk: int = 65536) -> np.ndarray:
        """[M, 2] predictions in target units."""
        X = features(q1, q2, undercooling, delta_a)
        outs = []
        for s in range(0, len(X), chunk):
            x16 = self.prepare(X[s:s + chunk])
            outs.append(self.forward(x16).cpu().numpy())
        self.check()
        return np.concatenate(outs) * self.std + self.mean

    def bf16_weights(self):
        """Host copies of the BF16 weights (as float64) and FP32 biases, per layer."""
        w16 = self.w16.cpu().numpy().view(np.uint16).astype(np.uint32) << 16
        wf = w16.view(np.float32).astype(np.float64)
        w = self.w.cpu().numpy().astype(np.float64)
        out = []
        for layer, (K, N, _) in enumerate(LAYERS):
            o, ob = self.offsets[layer]
            out.append((wf[o:o + N * K].reshape(N, K), w[ob:ob + N]))
        return out
