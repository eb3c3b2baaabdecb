"""Generate the golden vectors under ``tests/golden`` by running the reference's
own kernel sources (the 3D ``src/gpu_kernels_3d.py`` and the 2D
``src/gpu_kernels.py``) on the CPU through ``numba_typing_shim``
(compiled-Numba typing, serial grid loop).

Test infrastructure only.  Usage (needs a checkout of the reference)::

    python tests/golden/make_golden.py --reference /path/to/multiphasefield-solidification-v2

Inputs are built with the reference's own host helpers
(``src/seed_modes_3d.py``, ``src/orientation_utils.py``, ``src/seed_modes.py``)
imported from that checkout; the step sequence follows the reference's
drivers: ``tests/verification_3d.py:830-893`` (temperature, checked APT,
switchable update, swap), ``run_randommode_3d.py:267-287`` (temperature,
APT, update, swap) and, for the 2D kernels, ``tests/verification_3d.py:939-1000``
(run_2d_simulation).  Each case is written to ``<name>.npz``.
"""

from __future__ import annotations

import argparse
import math
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import numba_typing_shim as shim  # noqa: E402

KMAX = 50
MAX_GRAINS = 50

# config_3d.yaml values (reference), in SI units.
BASE = dict(dx=1.0e-4, dt=5.0e-5, T_melt=1687.0, G=1.0e2, V_pulling=5.0e-2, Sf=2.12e4,
            delta_factor=6.0, gamma_100=0.44, gamma_GB=0.60, a0_deg=54.7, delta_a=0.36,
            mu_a=0.6156, p_round=0.05, ksi=0.05, omg_deg=10.0, M_SL=5.0e-5, M_GB_ratio=0.07)

SCALAR_NAMES = ["dx", "dt", "T_melt", "Sf", "eps0_sl", "w0_sl", "a0", "delta_a", "mu_a",
                "p_round", "g2_floor", "ksi", "theta_c_rad"]


def derived(p):
    delta = p["delta_factor"] * p["dx"]
    eps = lambda g: math.sqrt(8.0 * delta * g / (math.pi * math.pi))
    w = lambda g: 4.0 * g / delta
    m = lambda mob: (math.pi * math.pi / (8.0 * delta)) * mob
    return dict(delta=delta, eps0_sl=eps(p["gamma_100"]), w0_sl=w(p["gamma_100"]),
                m_sl_phi=m(p["M_SL"]), eps_gb=eps(p["gamma_GB"]), w_gb=w(p["gamma_GB"]),
                m_gb_phi=m(p["M_SL"] * p["M_GB_ratio"]), a0=math.radians(p["a0_deg"]),
                theta_c_rad=math.radians(p["omg_deg"]), g2_floor=(0.1 / p["dx"]) ** 2,
                cooling_rate=p["G"] * p["V_pulling"] * p["dt"])


def scalars_of(p, d):
    return dict(dx=p["dx"], dt=p["dt"], T_melt=p["T_melt"], Sf=p["Sf"], eps0_sl=d["eps0_sl"],
                w0_sl=d["w0_sl"], a0=d["a0"], delta_a=p["delta_a"], mu_a=p["mu_a"],
                p_round=p["p_round"], g2_floor=d["g2_floor"], ksi=p["ksi"],
                theta_c_rad=d["theta_c_rad"])


def run_case(ref, name, phi0, temp0, quats, p, *, steps, f64, kernel="switchable",
             aniso=1, torque=1, checked=True, cooling=True, out_dir=HERE):
    om = ref["orientation_utils"]
    sm = ref["seed_modes"]
    K = ref["kernels"]
    d = derived(p)
    N, nx, ny, nz = phi0.shape
    n111 = om.compute_rotated_n111(quats).astype(np.float32)
    wij, aij, mij = sm.build_interaction_matrices(N, d["eps0_sl"], d["w0_sl"], d["m_sl_phi"],
                                                  d["eps_gb"], d["w_gb"], d["m_gb_phi"])
    wij, aij, mij = (a.astype(np.float32) for a in (wij, aij, mij))
    phi_dt = np.float64 if f64 else np.float32
    phi = phi0.astype(phi_dt).copy()
    phi_new = phi.copy()
    temp = temp0.copy()
    depth = max(MAX_GRAINS, KMAX, N)
    mf = np.zeros((depth, nx, ny, nz), np.int32)
    nf = np.zeros((nx, ny, nz), np.int32)
    status = np.zeros(2, np.int32)
    sc = scalars_of(p, d)
    scal32 = not f64
    sargs = [shim.scalar(sc[k], scal32) for k in SCALAR_NAMES]
    rate = shim.scalar(d["cooling_rate"], scal32)
    threads = (4, 4, 4)
    blocks = tuple(math.ceil(n / 4) for n in (nx, ny, nz))
    T = shim.TypedArray
    out = dict(phi0=phi0.astype(phi_dt), temp0=temp0.copy(), wij=wij, aij=aij, mij=mij,
               n111=n111, quats=quats, scalars=np.array([sc[k] for k in SCALAR_NAMES]),
               scalar_names=np.array(SCALAR_NAMES), scalars_f32=np.int32(scal32),
               cooling_rate=np.float64(d["cooling_rate"]), cooling=np.int32(cooling),
               kernel=np.array(kernel), aniso=np.int32(aniso), torque=np.int32(torque),
               checked=np.int32(checked), steps=np.int32(steps))
    phis, nfs, mfs, stats, temps = [], [], [], [], []
    t0 = time.time()
    for _ in range(steps):
        if cooling:
            K.kernel_update_temp_3d[blocks, threads](T(temp), rate, nx, ny, nz)
        status[:] = 0
        if checked:
            K.kernel_update_nfmf_3d_checked[blocks, threads](T(phi), T(mf), T(nf), T(status),
                                                              nx, ny, nz, N)
        else:
            K.kernel_update_nfmf_3d[blocks, threads](T(phi), T(mf), T(nf), nx, ny, nz, N)
        common = [T(phi), T(phi_new), T(temp), T(mf), T(nf), T(wij, read_as_f64=True), T(aij),
                  T(mij), T(n111), nx, ny, nz, N] + sargs
        if kernel == "switchable":
            K.kernel_update_phasefield_active_3d_switchable[blocks, threads](*common, aniso, torque)
        else:
            K.kernel_update_phasefield_active_3d[blocks, threads](*common)
        phi, phi_new = phi_new, phi
        phis.append(phi.copy())
        nfs.append(nf.copy())
        mfs.append(mf[: max(1, int(nf.max()))].copy())
        stats.append(status.copy())
        temps.append(temp.copy())
    out.update(phi=np.stack(phis), nf=np.stack(nfs), status=np.stack(stats),
               temp=np.stack(temps))
    dmax = max(m.shape[0] for m in mfs)
    mf_all = np.full((steps, dmax, nx, ny, nz), -1, np.int32)
    for s, m in enumerate(mfs):
        mf_all[s, : m.shape[0]] = m
    out["mf"] = mf_all
    np.savez_compressed(os.path.join(out_dir, f"{name}.npz"), **out)
    print(f"{name}: grid {nx}x{ny}x{nz} N={N} steps={steps} f64={f64} nf_max={int(nf.max())} "
          f"({time.time() - t0:.1f}s)")


def run_case_2d(ref, name, phi0, temp0, quats, p, *, steps, f64, out_dir=HERE):
    """Steps of the reference's 2D kernels in run_2d_simulation's order
    (tests/verification_3d.py:970-1000): temperature when the cooling rate is
    non-zero, APT, update, swap."""
    om = ref["orientation_utils"]
    sm = ref["seed_modes"]
    K = ref["kernels2d"]
    d = derived(p)
    N, nx, ny = phi0.shape
    n111 = om.compute_rotated_n111(quats).astype(np.float32)
    wij, aij, mij = sm.build_interaction_matrices(N, d["eps0_sl"], d["w0_sl"], d["m_sl_phi"],
                                                  d["eps_gb"], d["w_gb"], d["m_gb_phi"])
    wij, aij, mij = (a.astype(np.float32) for a in (wij, aij, mij))
    phi_dt = np.float64 if f64 else np.float32
    phi = phi0.astype(phi_dt).copy()
    phi_new = phi.copy()
    temp = temp0.copy()
    depth = max(20, N, 18)
    mf = np.zeros((depth, nx, ny), np.int32)
    nf = np.zeros((nx, ny), np.int32)
    sc = scalars_of(p, d)
    scal32 = not f64
    sargs = [shim.scalar(sc[k], scal32) for k in SCALAR_NAMES]
    rate = shim.scalar(d["cooling_rate"], scal32)
    threads = (4, 4)
    blocks = tuple(math.ceil(n / 4) for n in (nx, ny))
    T = shim.TypedArray
    out = dict(phi0=phi0.astype(phi_dt), temp0=temp0.copy(), wij=wij, aij=aij, mij=mij, n111=n111,
               quats=quats, scalars=np.array([sc[k] for k in SCALAR_NAMES]),
               scalar_names=np.array(SCALAR_NAMES), scalars_f32=np.int32(scal32),
               cooling_rate=np.float64(d["cooling_rate"]), steps=np.int32(steps))
    phis, nfs, mfs, temps = [], [], [], []
    t0 = time.time()
    for _ in range(steps):
        if d["cooling_rate"] != 0.0:
            K.kernel_update_temp[blocks, threads](T(temp), rate, nx, ny)
        K.kernel_update_nfmf[blocks, threads](T(phi), T(mf), T(nf), nx, ny, N)
        K.kernel_update_phasefield_active[blocks, threads](
            T(phi), T(phi_new), T(temp), T(mf), T(nf), T(wij, read_as_f64=True), T(aij), T(mij), T(n111),
            nx, ny, N, *sargs)
        phi, phi_new = phi_new, phi
        phis.append(phi.copy())
        nfs.append(nf.copy())
        mfs.append(mf[: max(1, int(nf.max()))].copy())
        temps.append(temp.copy())
    out.update(phi=np.stack(phis), nf=np.stack(nfs), temp=np.stack(temps))
    dmax = max(m.shape[0] for m in mfs)
    mf_all = np.full((steps, dmax, nx, ny), -1, np.int32)
    for s_, m in enumerate(mfs):
        mf_all[s_, : m.shape[0]] = m
    out["mf"] = mf_all
    np.savez_compressed(os.path.join(out_dir, f"{name}.npz"), **out)
    print(f"{name}: grid {nx}x{ny} N={N} steps={steps} f64={f64} nf_max={int(nf.max())} "
          f"({time.time() - t0:.1f}s)")


def stripes_phi_2d(nx, ny, n_solid, dx, delta, base, amp):
    """Solid stripes along x under a cosine front, liquid above (float32)."""
    x = np.arange(nx, dtype=np.float64).reshape(nx, 1)
    y = np.arange(ny, dtype=np.float64).reshape(1, ny)
    height = base + amp * np.cos(2.0 * math.pi * x / nx + 0.3)
    solid = (0.5 * (1.0 - np.tanh(np.float32(2.2 / delta) * (y - height) * dx))).astype(np.float32)
    phi = np.zeros((n_solid + 1, nx, ny), np.float32)
    edges = np.linspace(0, nx, n_solid + 1).astype(int)
    for g in range(1, n_solid + 1):
        phi[g, edges[g - 1]:edges[g], :] = solid[edges[g - 1]:edges[g], :]
    phi[0] = 1.0 - phi[1:].sum(axis=0)
    return phi


def apt_case(ref, name, phi, out_dir=HERE):
    K = ref["kernels"]
    N, nx, ny, nz = phi.shape
    depth = max(MAX_GRAINS, KMAX, N)
    mf = np.zeros((depth, nx, ny, nz), np.int32)
    nf = np.zeros((nx, ny, nz), np.int32)
    status = np.zeros(2, np.int32)
    T = shim.TypedArray
    blocks = tuple(math.ceil(n / 4) for n in (nx, ny, nz))
    K.kernel_update_nfmf_3d_checked[blocks, (4, 4, 4)](T(phi), T(mf), T(nf), T(status), nx, ny, nz, N)
    np.savez_compressed(os.path.join(out_dir, f"{name}.npz"), phi0=phi, mf=mf[: max(1, int(nf.max()))],
                        nf=nf, status=status)
    print(f"{name}: status={status.tolist()} nf_max={int(nf.max())}")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("MPF3D_REFERENCE_ROOT"),
                    required="MPF3D_REFERENCE_ROOT" not in os.environ,
                    help="checkout of the reference (or set MPF3D_REFERENCE_ROOT)")
    ap.add_argument("--only", default=None)
    args = ap.parse_args()
    sys.path.insert(0, args.reference)
    import importlib

    ref = dict(kernels=shim.load_reference_kernels(os.path.join(args.reference, "src", "gpu_kernels_3d.py")),
               kernels2d=shim.load_reference_kernels(os.path.join(args.reference, "src", "gpu_kernels.py"),
                                                     "reference_gpu_kernels_2d"),
               orientation_utils=importlib.import_module("src.orientation_utils"),
               seed_modes=importlib.import_module("src.seed_modes"),
               seed_modes_3d=importlib.import_module("src.seed_modes_3d"))
    s3 = ref["seed_modes_3d"]
    om = ref["orientation_utils"]
    p = dict(BASE)
    d = derived(p)
    want = lambda n: args.only is None or n in args.only.split(",")

    # Multi-grain Voronoi slab, undercooled (shape of verification case basic_constraints).
    nx, ny, nz = 10, 8, 12
    gmap = s3.generate_random_grain_map_3d(nx, ny, 4, random_seed=17)
    phi0 = s3.init_phi_from_grain_map_3d(gmap, 4, nx, ny, nz, p["dx"], d["delta"], 4)
    temp32 = np.full((nx, ny, nz), np.float32(p["T_melt"] - 5.0), np.float32)
    q4 = om.assign_quaternions_to_grains(4, mode="random", orientation_seed=23)
    if want("voronoi_f32"):
        run_case(ref, "voronoi_f32", phi0, temp32, q4, p, steps=3, f64=False)
    if want("voronoi_f64"):
        run_case(ref, "voronoi_f64", phi0, temp32.astype(np.float64), q4, p, steps=3, f64=True)

    # Production-driver sequence: unchecked APT, plain update kernel, float64 temperature
    # with a z gradient (run_randommode_3d.py).
    nx, ny, nz = 8, 8, 14
    gmap = s3.generate_random_grain_map_3d(nx, ny, 6, random_seed=5)
    phi0 = s3.init_phi_from_grain_map_3d(gmap, 6, nx, ny, nz, p["dx"], d["delta"], 5)
    temp = s3.init_temperature_field_3d(nx, ny, nz, p["T_melt"], 2.0e4, p["dx"], 5).astype(np.float64)
    q6 = om.assign_quaternions_to_grains(6, mode="random", orientation_seed=42)
    if want("driver_f32"):
        run_case(ref, "driver_f32", phi0, temp, q6, p, steps=3, f64=False, kernel="plain",
                 checked=False)
    if want("driver_f64"):
        run_case(ref, "driver_f64", phi0, temp, q6, p, steps=3, f64=True, kernel="plain",
                 checked=False)

    # Toggle coverage on a wavy single-grain front (anisotropy off; anisotropy on, torque off).
    nx, ny, nz = 12, 4, 12
    x = np.arange(nx, dtype=np.float64).reshape(nx, 1, 1)
    z = np.arange(nz, dtype=np.float64).reshape(1, 1, nz)
    height = 5.0 + 1.5 * np.cos(2.0 * math.pi * x / nx + 0.2)
    solid = (0.5 * (1.0 - np.tanh(np.float32(2.2 / d["delta"]) * (z - height) * p["dx"]))).astype(np.float32)
    wavy = np.zeros((2, nx, ny, nz), np.float32)
    wavy[1] = np.broadcast_to(solid, (nx, ny, nz))
    wavy[0] = 1.0 - wavy[1]
    qw = om.assign_quaternions_to_grains(1, mode="random", orientation_seed=7)
    tw = np.full((nx, ny, nz), np.float32(p["T_melt"] - 3.0), np.float32)
    pa = dict(p, delta_a=0.55, p_round=0.02)
    if want("wavy_iso_f32"):
        run_case(ref, "wavy_iso_f32", wavy, tw, qw, dict(p, ksi=1.0, delta_a=0.0), steps=3,
                 f64=False, aniso=0, torque=0)
    if want("wavy_notorque_f32"):
        run_case(ref, "wavy_notorque_f32", wavy, tw, qw, pa, steps=3, f64=False, aniso=1, torque=0)
    if want("wavy_aniso_f64"):
        run_case(ref, "wavy_aniso_f64", wavy, tw.astype(np.float64), qw, pa, steps=3, f64=True)

    # Grain junction: stripes meeting a tilted front, several active phases per cell.
    nx, ny, nz = 9, 6, 10
    gmap = np.zeros((nx, ny), np.int32)
    gmap[:3, :3], gmap[3:6, :3], gmap[6:, :3] = 1, 2, 3
    gmap[:3, 3:], gmap[3:6, 3:], gmap[6:, 3:] = 4, 5, 6
    phij = s3.init_phi_from_grain_map_3d(gmap, 6, nx, ny, nz, p["dx"], d["delta"], 4)
    qj = om.assign_quaternions_to_grains(6, mode="random", orientation_seed=99)
    tj = np.full((nx, ny, nz), p["T_melt"] - 2.0, np.float64)
    if want("junction_f64"):
        run_case(ref, "junction_f64", phij, tj, qj, p, steps=3, f64=True)
    if want("junction_f32"):
        run_case(ref, "junction_f32", phij, tj.astype(np.float32), qj, p, steps=3, f64=False)

    # 2D kernels.  two_d_limit_2d is the 2D half of two_d_limit_consistency
    # (tests/verification_3d.py:1509-1535): 12x14, one grain under a cosine
    # front at 4.8 +- 1.2 cells, delta_a = 0, ksi = 1, T_melt - 4, 6 steps.
    vparams = dict(p, delta_a=0.0, ksi=1.0)
    vd = derived(vparams)
    x = np.arange(12, dtype=np.float64).reshape(12, 1)
    y = np.arange(14, dtype=np.float64).reshape(1, 14)
    h2 = 4.8 + 1.2 * np.cos(2.0 * math.pi * x / 12)
    s2 = (0.5 * (1.0 - np.tanh(np.float32(2.2 / vd["delta"]) * (y - h2) * p["dx"]))).astype(np.float32)
    phi2 = np.zeros((2, 12, 14), np.float32)
    phi2[1] = s2
    phi2[0] = 1.0 - phi2[1]
    qid = np.array([[0.0, 0.0, 0.0, 1.0], [0.0, 0.0, 0.0, 1.0]])
    if want("two_d_limit_2d"):
        run_case_2d(ref, "two_d_limit_2d", phi2, np.full((12, 14), np.float32(p["T_melt"] - 4.0), np.float32),
                    qid, vparams, steps=6, f64=False)
    # Anisotropic multi-grain 2D fronts: three stripes meeting a wavy front.
    phis = stripes_phi_2d(15, 12, 3, p["dx"], d["delta"], 5.0, 1.5)
    q3 = om.assign_quaternions_to_grains(3, mode="random", orientation_seed=31)
    t2 = np.full((15, 12), np.float32(p["T_melt"] - 3.0), np.float32)
    if want("stripes2d_f32"):
        run_case_2d(ref, "stripes2d_f32", phis, t2, q3, p, steps=3, f64=False)
    if want("stripes2d_f64"):
        run_case_2d(ref, "stripes2d_f64", phis, t2.astype(np.float64), q3, dict(p, p_round=0.02), steps=3,
                    f64=True)

    # Grain-boundary groove: the set-up of groove_depth_only / robust_groove_angle_estimation
    # (tests/verification_3d.py:2453-2489, 2491-2539): 20x6x24 bicrystal under a front at
    # 7 + 0.6 cos(2 pi x/nx), isotropic (delta_a 0, ksi 1, both toggles off), G = V = 0,
    # T_melt, 20 steps.  The reference's recorded groove metrics of this run pin the analysis.
    if want("groove_f32"):
        bi = importlib.import_module("bicrystal_reference")
        pg = dict(p, delta_a=0.0, ksi=1.0, G=0.0, V_pulling=0.0)
        dg = derived(pg)
        phig = bi.reference_functions(args.reference)["bicrystal_phi_3d"](
            20, 6, 24, pg["dx"], dg["delta"], 7.0, 10, waviness=0.6)
        qg = np.array([[0.0, 0.0, 0.0, 1.0]] * 3)
        tg = np.full((20, 6, 24), np.float32(pg["T_melt"]), np.float32)
        run_case(ref, "groove_f32", phig, tg, qg, pg, steps=20, f64=False, aniso=0, torque=0,
                 cooling=False)

    # APT known answers: boundary probes and the crafted KMAX overflow
    # (tests/verification_3d.py:1459-1480, 1538-1565).
    if want("apt_boundary"):
        pb = np.zeros((4, 6, 5, 5), np.float32)
        pb[1, 0, 2, 2] = 1.0
        pb[2, 3, 0, 2] = 1.0
        pb[3, 3, 2, 0] = 1.0
        pb[0] = np.clip(1.0 - pb[1:].sum(axis=0), 0.0, 1.0)
        apt_case(ref, "apt_boundary", pb)
    if want("apt_overflow"):
        n = KMAX + 2
        po = np.zeros((n, 4, 4, 4), np.float32)
        po[:, 1, 1, 1] = np.float32(1.0 / n)
        po[0] = np.clip(1.0 - po[1:].sum(axis=0), 0.0, 1.0)
        apt_case(ref, "apt_overflow", po)


if __name__ == "__main__":
    main()
