"""The numerical method of the compact tier's facet angle (facet_angle in
csrc/compact.cu), restated step for step in numpy float32 with explicit
roundings and fused multiply-adds, against the float64 acos that the
reference evaluates (calc_b_from_cos, src/gpu_kernels_3d.py:33-55, on the
float32 rotated normals of src/orientation_utils.py:182-212).  Near a facet
the direct FP32 acos of the best |cos| loses most of theta; the
reformulation keeps theta to ~3e-8 rad and b(theta) to ~1e-6 relative."""
import math

import numpy as np

f32 = np.float32
THETA_C = math.radians(10.0)


def fma(a, b, c):
    """float32 fused multiply-add: the float64 product of two float32 values
    is exact, so one rounding of the float64 sum is one rounding in total
    up to a double-rounding tie."""
    return f32(np.float64(a) * np.float64(b) + np.float64(c))


def diff_of_products(a, b, c, d):
    w = f32(c * d)
    e = fma(-c, d, w)
    f = fma(a, b, -w)
    return f32(f + e)


def facet_angle(g, n):
    """theta = acos(|g . n| / |g|) from 1 - c = (1 - |n|) + (1 - cos t)."""
    gx, gy, gz = (f32(v) for v in g)
    nx, ny, nz = (f32(v) for v in n)
    q = f32(f32(f32(gx * gx) + f32(gy * gy)) + f32(gz * gz))
    p1, p2, p3 = f32(nx * nx), f32(ny * ny), f32(nz * nz)
    e1, e2, e3 = fma(nx, nx, -p1), fma(ny, ny, -p2), fma(nz, nz, -p3)
    s1 = f32(p1 + p2)
    t1 = f32(s1 - p1)
    err = f32(f32(p1 - f32(s1 - t1)) + f32(p2 - t1))
    s2 = f32(s1 + p3)
    t2 = f32(s2 - s1)
    err = f32(err + f32(f32(s1 - f32(s2 - t2)) + f32(p3 - t2)))
    dn2 = f32(f32(f32(1) - s2) - f32(err + f32(e1 + f32(e2 + e3))))
    cx = diff_of_products(gy, nz, gz, ny)
    cy = diff_of_products(gz, nx, gx, nz)
    cz = diff_of_products(gx, ny, gy, nx)
    sin2 = f32(f32(f32(f32(cx * cx) + f32(cy * cy)) + f32(cz * cz)) / f32(q * f32(1 - dn2)))
    ig = f32(1) / np.sqrt(q)
    cabs = min(abs(f32(f32(f32(gx * ig) * nx) + f32(f32(gy * ig) * ny)) + f32(f32(gz * ig) * nz)), f32(1))
    omc = max(f32(f32(f32(0.5) * dn2) + f32(sin2 / f32(f32(1) + cabs))), f32(0))
    return f32(2) * np.arcsin(np.sqrt(f32(0.5) * omc))


def direct_fp32_angle(g, n):
    g32 = np.asarray(g, f32)
    q = f32((g32 * g32).sum(dtype=f32))
    c = min(abs(f32((g32 * (f32(1) / np.sqrt(q))) @ np.asarray(n, f32))), f32(1))
    return np.arccos(c)


def b_of(theta, ksi=0.01):
    if theta >= THETA_C:
        return 1.0
    y = min(max(0.5 * math.pi * theta / THETA_C, 1e-6), 0.5 * math.pi - 1e-6)
    t = math.tan(y)
    return ksi + (1.0 - ksi) * t * math.tanh(1.0 / t)


def near_facet_samples(n_samples, seed):
    rng = np.random.default_rng(seed)
    base = np.array([1.0, 1.0, 1.0]) / math.sqrt(3.0)
    for _ in range(n_samples):
        rot = np.linalg.qr(rng.normal(size=(3, 3)))[0]
        n32 = (rot @ base).astype(f32)
        n = n32.astype(np.float64)
        th = 10 ** rng.uniform(-6, math.log10(THETA_C))
        perp = np.cross(n, rng.normal(size=3))
        perp /= np.linalg.norm(perp)
        g32 = ((math.cos(th) * n + math.sin(th) * perp) * 10 ** rng.uniform(3, 5) * rng.choice([-1, 1])).astype(f32)
        g = g32.astype(np.float64)
        theta64 = math.acos(min(abs(g @ n) / np.linalg.norm(g), 1.0))
        yield g32, n32, theta64


def test_reformulated_angle_tracks_float64_acos_near_facets():
    worst_theta = worst_b = 0.0
    for g, n, theta64 in near_facet_samples(4000, seed=11):
        theta = float(facet_angle(g, n))
        worst_theta = max(worst_theta, abs(theta - theta64))
        worst_b = max(worst_b, abs(b_of(theta) - b_of(theta64)) / b_of(theta64))
    assert worst_theta < 1e-7
    assert worst_b < 2e-6


def test_direct_fp32_acos_is_ill_conditioned_there():
    """The formulation it replaces: relative errors in b of several percent."""
    worst_b = 0.0
    for g, n, theta64 in near_facet_samples(4000, seed=11):
        theta = float(direct_fp32_angle(g, n))
        worst_b = max(worst_b, abs(b_of(theta) - b_of(theta64)) / b_of(theta64))
    assert worst_b > 1e-2


def test_normal_longer_than_one_clamps_to_zero_angle():
    """c > 1 (|n| > 1 after rounding, g along n) gives theta = 0, as the
    reference's clamp of c to 1 does."""
    n = np.array([0.5773503, 0.5773503, 0.5773503], f32)  # |n|^2 slightly above 1 in float32
    g = n.astype(np.float64) * 1e4
    assert float(facet_angle(g, n)) == 0.0
