"""Surrogate network kernels on the GPU: the BF16 tensor-core GEMMs against a
float64 product of the same BF16 operands (all operand layouts the network
uses, forward and gradients on tcgen05), the full backward pass against a
CPU float64 restatement with the same BF16 rounding points, and training on
a smooth target."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def bf16_round(x):
    """Round float values to BF16 (nearest even), returned as float64."""
    u = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return (u.astype(np.uint32) << 16).view(np.float32).astype(np.float64)


def to_bf16_bits(x):
    u = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    return ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16).view(np.int16)


@pytest.mark.parametrize("M,N,K,transA,transB", [(100, 70, 40, False, False), (64, 256, 16, False, True),
                                                 (256, 16, 300, True, False), (33, 2, 256, False, True)])
def test_gemm_matches_float64(M, N, K, transA, transB):
    from mpf3d import _lib
    rng = np.random.default_rng(M + N + K)
    A = rng.standard_normal((M, K)).astype(np.float32)
    B = rng.standard_normal((K, N)).astype(np.float32)
    bias = rng.standard_normal(N).astype(np.float32)
    A_store = A.T.copy() if transA else A
    B_store = B.T.copy() if transB else B
    sam, sak = (1, M) if transA else (K, 1)
    sbk, sbn = (1, K) if transB else (N, 1)
    dev = torch.device("cuda:0")
    tA = torch.from_numpy(to_bf16_bits(A_store)).to(dev)
    tB = torch.from_numpy(to_bf16_bits(B_store)).to(dev)
    tb = torch.from_numpy(bias).to(dev)
    Y = torch.empty((M, N), dtype=torch.float32, device=dev)
    Z = torch.empty((M, N), dtype=torch.float32, device=dev)
    rc = _lib.lib().mpf3d_gemm_bf16(M, N, K, tA.data_ptr(), sam, sak, tB.data_ptr(), sbk, sbn, tb.data_ptr(), 1,
                                    Z.data_ptr(), Y.data_ptr(), N, 0, 0, None, None)
    assert rc == 0
    ref_z = bf16_round(A) @ bf16_round(B) + bias
    ref_y = ref_z / (1.0 + np.exp(-ref_z))
    got_z = Z.cpu().numpy()
    got_y = Y.cpu().numpy()
    scale = np.abs(ref_z).max()
    assert np.abs(got_z - ref_z).max() <= 1e-5 * scale * np.sqrt(K)
    assert np.abs(got_y - ref_y).max() <= 1e-3 * scale


@pytest.mark.parametrize("M,N,K,act,y_bf16", [(300, 256, 256, 1, 1), (128, 256, 16, 1, 0), (77, 16, 256, 0, 0),
                                             (1000, 128, 64, 1, 1), (129, 2, 256, 0, 0), (256, 200, 32, 0, 0),
                                             (513, 96, 192, 1, 0), (40000, 256, 128, 1, 1)])
def test_tcgen05_gemm_matches_float64(M, N, K, act, y_bf16):
    """The tensor-memory kernels (K-major X [M][K], W [N][K]; TMA-fed and
    pipelined for K a multiple of 64, staged through registers otherwise)
    against a float64 product of the same BF16 operands, and against the
    mma.sync kernel."""
    from mpf3d import _lib
    rng = np.random.default_rng(M * 7 + N + K)
    X = rng.standard_normal((M, K)).astype(np.float32)
    W = rng.standard_normal((N, K)).astype(np.float32)
    bias = rng.standard_normal(N).astype(np.float32)
    dev = torch.device("cuda:0")
    tX = torch.from_numpy(to_bf16_bits(X)).to(dev)
    tW = torch.from_numpy(to_bf16_bits(W)).to(dev)
    tb = torch.from_numpy(bias).to(dev)
    ydt = torch.int16 if y_bf16 else torch.float32
    Z = torch.full((M, N), float("nan"), dtype=torch.float32, device=dev)
    Y = torch.zeros((M, N), dtype=ydt, device=dev)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    rc = _lib.lib().mpf3d_gemm_bf16_tc5(M, N, K, tX.data_ptr(), K, tW.data_ptr(), K, tb.data_ptr(), act,
                                        Z.data_ptr(), Y.data_ptr(), N, y_bf16, 0, err.data_ptr(), None)
    assert rc == 0
    assert int(err.item()) == 0
    ref_z = bf16_round(X) @ bf16_round(W).T + bias
    got_z = Z.cpu().numpy()
    scale = np.abs(ref_z).max()
    assert np.isfinite(got_z).all()
    assert np.abs(got_z - ref_z).max() <= 1e-5 * scale * np.sqrt(K)
    Z2 = torch.empty((M, N), dtype=torch.float32, device=dev)
    Y2 = torch.zeros((M, N), dtype=ydt, device=dev)
    rc = _lib.lib().mpf3d_gemm_bf16_mma(M, N, K, tX.data_ptr(), K, 1, tW.data_ptr(), 1, K, tb.data_ptr(), act,
                                        Z2.data_ptr(), Y2.data_ptr(), N, y_bf16, 0, None)
    assert rc == 0
    assert np.abs(Z2.cpu().numpy() - got_z).max() <= 1e-5 * scale * np.sqrt(K)
    if y_bf16:
        ya = (Y.cpu().numpy().view(np.uint16).astype(np.uint32) << 16).view(np.float32)
        yb = (Y2.cpu().numpy().view(np.uint16).astype(np.uint32) << 16).view(np.float32)
        assert np.abs(ya - yb).max() <= 1e-2 * max(1.0, np.abs(yb).max())
    else:
        assert np.abs(Y.cpu().numpy() - Y2.cpu().numpy()).max() <= 1e-4 * scale * np.sqrt(K)


@pytest.mark.parametrize("M,N,K,transA,transB,beta", [(256, 256, 600, True, False, 0), (2, 256, 512, True, False, 1),
                                                      (512, 256, 2, False, True, 0), (300, 16, 256, True, False, 0),
                                                      (512, 256, 256, False, True, 1), (77, 200, 40, True, True, 0)])
def test_tcgen05_gradient_gemm_matches_float64(M, N, K, transA, transB, beta):
    """The tcgen05 kernel for transposed operands (the surrogate's gradients:
    dW = dZ^T X with the batch as reduction, dH = dZ W with W read across its
    rows), against a float64 product of the same BF16 operands: reductions
    deeper than one 256-deep block (accumulated block by block), reductions
    padded to a multiple of 16, and accumulation into the output (beta)."""
    from mpf3d import _lib
    rng = np.random.default_rng(M * 3 + N + K)
    A = rng.standard_normal((M, K)).astype(np.float32)
    B = rng.standard_normal((K, N)).astype(np.float32)
    A_store = A.T.copy() if transA else A
    B_store = B.T.copy() if transB else B
    sam, sak = (1, M) if transA else (K, 1)
    sbk, sbn = (1, K) if transB else (N, 1)
    dev = torch.device("cuda:0")
    tA = torch.from_numpy(to_bf16_bits(A_store)).to(dev)
    tB = torch.from_numpy(to_bf16_bits(B_store)).to(dev)
    Y0 = rng.standard_normal((M, N)).astype(np.float32)
    Y = torch.from_numpy(Y0.copy()).to(dev)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    rc = _lib.lib().mpf3d_gemm_bf16_tc5_strided(M, N, K, tA.data_ptr(), sam, sak, tB.data_ptr(), sbk, sbn, None, 0,
                                                None, Y.data_ptr(), N, 0, beta, err.data_ptr(), None)
    assert rc == 0
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    ref = bf16_round(A) @ bf16_round(B) + (Y0 if beta else 0.0)
    scale = np.abs(bf16_round(A) @ bf16_round(B)).max()
    assert np.abs(Y.cpu().numpy() - ref).max() <= 1e-5 * scale * np.sqrt(K)


def test_tcgen05_rejects_shapes_it_does_not_cover():
    from mpf3d import _lib
    L = _lib.lib()
    p = 0x10000
    assert L.mpf3d_gemm_bf16_tc5(64, 300, 64, p, 64, p, 64, None, 0, None, p, 300, 0, 0, None, None) == -1  # N > 256
    assert L.mpf3d_gemm_bf16_tc5(64, 64, 24, p, 24, p, 24, None, 0, None, p, 64, 0, 0, None, None) == -1    # K % 16
    assert L.mpf3d_gemm_bf16_tc5(64, 64, 512, p, 512, p, 512, None, 0, None, p, 64, 0, 0, None, None) == -1  # K > 256
    # a reduction deeper than 256 accumulates into FP32: no activation, no Z, no BF16 output
    assert L.mpf3d_gemm_bf16_tc5_strided(64, 64, 512, p, 1, 64, p, 1, 512, None, 1, None, p, 64, 0, 0, None,
                                         None) == -1
    assert L.mpf3d_gemm_bf16_tc5_strided(64, 64, 512, p, 1, 64, p, 1, 512, None, 0, None, p, 64, 1, 0, None,
                                         None) == -1


def test_tcgen05_abort_path_reports_and_frees():
    """The pipelined kernel with its TMA producer held back: no copy and no
    MMA is ever issued, so every bounded wait of the MMA and epilogue roles
    runs out (after 20 ms).  The kernel must report MPF3D_DEV_GEMM_ABORT,
    write NaN, free its tensor memory and leave the context usable: an
    ordinary GEMM right after it gives the right answer twice."""
    from mpf3d import _lib
    L = _lib.lib()
    M, N, K = 512, 128, 64
    rng = np.random.default_rng(3)
    X = rng.standard_normal((M, K)).astype(np.float32)
    W = rng.standard_normal((N, K)).astype(np.float32)
    dev = torch.device("cuda:0")
    tX = torch.from_numpy(to_bf16_bits(X)).to(dev)
    tW = torch.from_numpy(to_bf16_bits(W)).to(dev)
    Y = torch.zeros((M, N), dtype=torch.float32, device=dev)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    assert L.mpf3d_gemm_bf16_tc5_held(M, N, K, tX.data_ptr(), K, tW.data_ptr(), K, Y.data_ptr(), N,
                                      err.data_ptr(), 20_000_000, None) == 0
    torch.cuda.synchronize()
    assert int(err.item()) & 32
    assert torch.isnan(Y).all()
    ref = bf16_round(X) @ bf16_round(W).T
    for _ in range(2):
        err.zero_()
        Y.zero_()
        assert L.mpf3d_gemm_bf16_tc5(M, N, K, tX.data_ptr(), K, tW.data_ptr(), K, None, 0, None, Y.data_ptr(), N, 0,
                                     0, err.data_ptr(), None) == 0
        torch.cuda.synchronize()
        assert int(err.item()) == 0
        assert np.abs(Y.cpu().numpy() - ref).max() <= 1e-5 * np.abs(ref).max() * np.sqrt(K)


def cpu_forward_backward(layers, X, target, w):
    """Float64 restatement of Surrogate.forward/backward with the GPU's BF16
    rounding points: hidden activations and the dZ operands of the GEMMs are
    BF16, pre-activations and accumulations exact."""
    silu = lambda z: z / (1.0 + np.exp(-z))
    dsilu = lambda z: (1 / (1 + np.exp(-z))) * (1 + z * (1 - 1 / (1 + np.exp(-z))))
    hs, zs = [X], []
    h = X
    for i, (W, b) in enumerate(layers):
        z = h @ W.T + b
        zs.append(z)
        h = z if i == len(layers) - 1 else bf16_round(silu(z))
        hs.append(h)
    out = h
    M = X.shape[0]
    dY = 2.0 * w * (out - target) / M
    grads = []
    for i in range(len(layers) - 1, -1, -1):
        W, b = layers[i]
        dZ = dY if i == len(layers) - 1 else dY * dsilu(zs[i])
        dZ16 = bf16_round(dZ)
        grads.append((dZ16.T @ hs[i], dZ.sum(0)))
        dY = dZ16 @ W
    return out, grads[::-1]


def test_backward_matches_cpu_float64_restatement():
    from mpf3d.surrogate import Surrogate, LAYERS, IN_FEATURES, DERIVED, HIDDEN, K1
    s = Surrogate(seed=3)
    rng = np.random.default_rng(0)
    M = 96
    X = rng.uniform(-1, 1, (M, IN_FEATURES + DERIVED)).astype(np.float32)
    T = rng.standard_normal((M, 2)).astype(np.float32)
    x16 = s.prepare(X)
    tT = torch.from_numpy(T).to("cuda:0")
    s.loss_and_grad(x16, tT)
    g = s.g.cpu().numpy().astype(np.float64)
    layers = s.bf16_weights()
    Xp = np.zeros((M, K1))
    Xp[:, :IN_FEATURES + DERIVED] = bf16_round(X)
    out, grads = cpu_forward_backward(layers, Xp, T.astype(np.float64), np.ones(2))
    gpu_out = s.forward(x16).cpu().numpy()
    assert np.abs(gpu_out - out).max() <= 2e-2 * max(1.0, np.abs(out).max())
    for layer, (K, N, _) in enumerate(LAYERS):
        o, ob = s.offsets[layer]
        gW = g[o:o + N * K].reshape(N, K)
        gb = g[ob:ob + N]
        rW, rb = grads[layer]
        if layer == 0:
            rW = rW.copy()
            rW[:, IN_FEATURES + DERIVED:] = 0.0
        for got, ref in ((gW, rW), (gb, rb)):
            err = np.linalg.norm(got - ref) / max(np.linalg.norm(ref), 1e-12)
            assert err <= 2e-2, f"layer {layer}: relative gradient error {err:.3e}"


def test_training_fits_a_smooth_target():
    from mpf3d.surrogate import Surrogate
    rng = np.random.default_rng(1)
    n = 512
    q1 = rng.standard_normal((n, 4))
    q1 /= np.linalg.norm(q1, axis=1, keepdims=True)
    q2 = rng.standard_normal((n, 4))
    q2 /= np.linalg.norm(q2, axis=1, keepdims=True)
    dT = rng.uniform(0.25, 3.0, n)
    da = rng.uniform(0, 1, n)
    y = np.stack([np.sin(2 * dT) + da, dT * da - 0.5], 1)
    s = Surrogate(seed=0)
    hist = s.fit(q1, q2, dT, da, y, epochs=150, batch=128, lr=3e-3, augment_symmetry=False)
    assert hist[-1] < 0.05 * hist[0]
    pred = s.predict(q1, q2, dT, da)
    assert np.sqrt(np.mean((pred - y) ** 2)) < 0.1
