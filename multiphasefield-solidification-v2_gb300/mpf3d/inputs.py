"""Host-side inputs of the 3D step: derived constants, interaction matrices,
rotated {111} normals, grain quaternions and initial fields.

These restate the reference's host helpers so that tests and benchmarks run
where the reference is not installed:
  derived constants      run_randommode_3d.py:56-65, 179-184, 260-263;
                         tests/verification_3d.py:177-204
  interaction matrices   src/seed_modes.py:333-380
  rotated {111} normals  src/orientation_utils.py:182-212
  random quaternions     src/orientation_utils.py:152-156
  tanh front / fields    src/seed_modes_3d.py:27-57
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

# config_3d.yaml of the reference (SI units)
CONFIG_3D = dict(dx=1.0e-4, dt=5.0e-5, T_melt=1687.0, G=1.0e2, V_pulling=5.0e-2, Sf=2.12e4,
                 delta_factor=6.0, gamma_100=0.44, gamma_GB=0.60, a0_deg=54.7, delta_a=0.36,
                 mu_a=0.6156, p_round=0.05, ksi=0.05, omg_deg=10.0, M_SL=5.0e-5, M_GB_ratio=0.07)


@dataclass
class Physics:
    """Physical and numerical parameters (config_3d.yaml keys)."""
    dx: float = 1.0e-4
    dt: float = 5.0e-5
    T_melt: float = 1687.0
    G: float = 1.0e2
    V_pulling: float = 5.0e-2
    Sf: float = 2.12e4
    delta_factor: float = 6.0
    gamma_100: float = 0.44
    gamma_GB: float = 0.60
    a0_deg: float = 54.7
    delta_a: float = 0.36
    mu_a: float = 0.6156
    p_round: float = 0.05
    ksi: float = 0.05
    omg_deg: float = 10.0
    M_SL: float = 5.0e-5
    M_GB_ratio: float = 0.07

    def replace(self, **kw) -> "Physics":
        d = dict(self.__dict__)
        d.update(kw)
        return Physics(**d)

    def derived(self) -> dict:
        delta = self.delta_factor * self.dx
        eps = lambda g: math.sqrt(8.0 * delta * g / (math.pi * math.pi))
        w = lambda g: 4.0 * g / delta
        m = lambda mob: (math.pi * math.pi / (8.0 * delta)) * mob
        return dict(delta=delta, eps0_sl=eps(self.gamma_100), w0_sl=w(self.gamma_100),
                    m_sl_phi=m(self.M_SL), eps_gb=eps(self.gamma_GB), w_gb=w(self.gamma_GB),
                    m_gb_phi=m(self.M_SL * self.M_GB_ratio), a0=math.radians(self.a0_deg),
                    theta_c_rad=math.radians(self.omg_deg), g2_floor=(0.1 / self.dx) ** 2,
                    cooling_rate=self.G * self.V_pulling * self.dt)

    def kernel_scalars(self, f32: bool = True) -> tuple:
        """The 13 float arguments of the reference's update kernel, typed as
        its drivers pass them (np.float32) or as float64."""
        d = self.derived()
        vals = (self.dx, self.dt, self.T_melt, self.Sf, d["eps0_sl"], d["w0_sl"], d["a0"],
                self.delta_a, self.mu_a, self.p_round, d["g2_floor"], self.ksi, d["theta_c_rad"])
        cast = np.float32 if f32 else np.float64
        return tuple(cast(v) for v in vals)


def interaction_matrices(N: int, eps0_sl, w0_sl, m_sl_phi, eps_gb, w_gb, m_gb_phi):
    """wij, aij, mij [N, N] float32: solid-solid pairs get the grain-boundary
    values, solid-liquid pairs the solid-liquid baselines, the diagonal 0."""
    wij = np.zeros((N, N), np.float32)
    aij = np.zeros((N, N), np.float32)
    mij = np.zeros((N, N), np.float32)
    if N > 1:
        s = slice(1, N)
        wij[s, s] = w_gb
        aij[s, s] = eps_gb
        mij[s, s] = m_gb_phi
        idx = np.arange(1, N)
        wij[idx, idx] = 0.0
        aij[idx, idx] = 0.0
        mij[idx, idx] = 0.0
        wij[0, s] = wij[s, 0] = w0_sl
        aij[0, s] = aij[s, 0] = eps0_sl
        mij[0, s] = mij[s, 0] = m_sl_phi
    return wij, aij, mij


def matrices_for(phys: Physics, N: int):
    d = phys.derived()
    return interaction_matrices(N, d["eps0_sl"], d["w0_sl"], d["m_sl_phi"], d["eps_gb"], d["w_gb"],
                                d["m_gb_phi"])


def random_quaternions(n_solid: int, seed: int) -> np.ndarray:
    """[n_solid+1, 4] (x, y, z, w); row 0 is the liquid's identity.  Each grain
    draws 4 standard normals from one default_rng(seed) stream and normalises."""
    q = np.zeros((n_solid + 1, 4), np.float64)
    q[0] = (0.0, 0.0, 0.0, 1.0)
    rng = np.random.default_rng(seed)
    for g in range(1, n_solid + 1):
        v = rng.standard_normal(4)
        q[g] = v / np.linalg.norm(v)
    return q


def _quat_to_matrix(q: np.ndarray) -> np.ndarray:
    x, y, z, w = q / np.linalg.norm(q)
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def rotated_n111(quats: np.ndarray) -> np.ndarray:
    """[N, 8, 3] float32: the 8 {111} normals (+-1,+-1,+-1)/sqrt(3) rotated by
    each grain's quaternion (scalar-last convention)."""
    base = np.array([[1, 1, 1], [1, 1, -1], [1, -1, 1], [-1, 1, 1], [1, -1, -1], [-1, 1, -1],
                     [-1, -1, 1], [-1, -1, -1]], np.float64) / math.sqrt(3.0)
    out = np.zeros((quats.shape[0], 8, 3), np.float32)
    for g, q in enumerate(quats):
        R = _quat_to_matrix(np.asarray(q, np.float64)).astype(np.float32).astype(np.float64)
        out[g] = (R @ base.T).T
    return out


def tanh_profile(nz: int, height: float, dx: float, delta: float) -> np.ndarray:
    """Solid fraction along z: 0.5 * (1 - tanh(2.2/delta * (k - height) * dz))."""
    k = np.arange(nz, dtype=np.float64)
    return (0.5 * (1.0 - np.tanh(np.float32(2.2 / delta) * (k - height) * dx))).astype(np.float32)


def temperature_field(nx, ny, nz, T_melt, G, dz, seed_height, dtype=np.float32) -> np.ndarray:
    """T(k) = T_melt + G * (k - seed_height) * dz, broadcast over x, y."""
    k = np.arange(nz, dtype=np.float64)
    t1 = (T_melt + G * (k - seed_height) * dz).astype(np.float32)
    return np.broadcast_to(t1[None, None, :], (nx, ny, nz)).astype(dtype).copy()


def voronoi_slab_owner(nx, ny, nz, n_grains, slab, seed) -> np.ndarray:
    """[nx, ny, nz] int32 grain id 1..n_grains: nearest of n_grains seed points
    drawn uniformly in the bottom `slab` z-layers (periodic in x and y)."""
    from scipy.spatial import cKDTree

    rng = np.random.default_rng(seed)
    sx = rng.uniform(0, nx, n_grains)
    sy = rng.uniform(0, ny, n_grains)
    sz = rng.uniform(0, slab, n_grains)
    big = 4.0 * (nx + ny + nz + slab)
    tree = cKDTree(np.stack([sx, sy, sz], 1) % [nx, ny, big], boxsize=[nx, ny, big])
    ks = min(slab, nz)
    gx, gy, gz = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(ks), indexing="ij")
    _, idx = tree.query(np.stack([gx.ravel(), gy.ravel(), gz.ravel()], 1).astype(np.float64), workers=-1)
    owner = np.empty((nx, ny, nz), np.int32)
    owner[:, :, :ks] = (idx.reshape(nx, ny, ks) + 1).astype(np.int32)
    if nz > ks:
        owner[:, :, ks:] = owner[:, :, ks - 1:ks]
    return owner


def phi_from_owner(owner: np.ndarray, n_grains: int, profile: np.ndarray, dtype=np.float32):
    """Dense phi [n_grains+1, nx, ny, nz]: grain g holds the z profile where it
    owns the cell; liquid = clip(1 - sum of solids, 0, 1)."""
    nx, ny, nz = owner.shape
    phi = np.zeros((n_grains + 1, nx, ny, nz), dtype)
    prof = np.broadcast_to(profile[None, None, :], (nx, ny, nz))
    for g in range(1, n_grains + 1):
        phi[g] = np.where(owner == g, prof, 0.0)
    phi[0] = np.clip(1.0 - phi[1:].sum(axis=0, dtype=np.float32), 0.0, 1.0)
    return phi


@dataclass
class Case:
    """A complete set of step inputs on the host."""
    phi: np.ndarray
    temp: np.ndarray
    quats: np.ndarray
    n111: np.ndarray
    wij: np.ndarray
    aij: np.ndarray
    mij: np.ndarray
    phys: Physics = field(default_factory=Physics)


def voronoi_case(nx, ny, nz, n_grains, slab, seed=0, orientation_seed=1, phys: Physics | None = None,
                 undercooling=None, dtype=np.float32) -> Case:
    """3D Voronoi slab of n_grains grains under a tanh front at z = slab;
    temperature from the config gradient, or uniform T_melt - undercooling."""
    phys = phys or Physics()
    d = phys.derived()
    owner = voronoi_slab_owner(nx, ny, nz, n_grains, slab, seed)
    prof = tanh_profile(nz, slab, phys.dx, d["delta"])
    phi = phi_from_owner(owner, n_grains, prof, dtype)
    if undercooling is None:
        temp = temperature_field(nx, ny, nz, phys.T_melt, phys.G, phys.dx, slab)
    else:
        temp = np.full((nx, ny, nz), np.float32(phys.T_melt - undercooling), np.float32)
    q = random_quaternions(n_grains, orientation_seed)
    wij, aij, mij = matrices_for(phys, n_grains + 1)
    return Case(phi, temp, q, rotated_n111(q), wij, aij, mij, phys)


def grain_map_2d(nx: int, ny: int, n_solid: int, seed: int) -> np.ndarray:
    """[nx, ny] int32 grain ids 1..n_solid: nearest of n_solid seed points
    drawn uniformly in the x-y plane from default_rng(seed) (x coordinates
    first, then y); the columnar map of generate_random_grain_map_3d,
    src/seed_modes_3d.py:15-24."""
    rng = np.random.default_rng(seed)
    sx = rng.uniform(0, nx, n_solid).reshape(-1, 1, 1)
    sy = rng.uniform(0, ny, n_solid).reshape(-1, 1, 1)
    lx = np.arange(nx, dtype=np.float32).reshape(1, nx, 1)
    ly = np.arange(ny, dtype=np.float32).reshape(1, 1, ny)
    return (np.argmin((lx - sx) ** 2 + (ly - sy) ** 2, axis=0) + 1).astype(np.int32)


def phi_from_grain_map_2d(gmap: np.ndarray, n_solid: int, nz: int, dz: float, delta: float, height: float):
    """Columnar phi [n_solid+1, nx, ny, nz]: each column's grain holds the tanh
    profile of the front at `height` (init_phi_from_grain_map_3d,
    src/seed_modes_3d.py:38-57)."""
    nx, ny = gmap.shape
    prof = tanh_profile(nz, height, dz, delta)
    phi = np.zeros((n_solid + 1, nx, ny, nz), np.float32)
    for g in range(1, n_solid + 1):
        phi[g] = np.where((gmap == g)[:, :, None], prof[None, None, :], 0.0)
    phi[0] = np.clip(1.0 - phi[1:].sum(axis=0), 0.0, 1.0)
    return phi


def wavy_front(nx: int, ny: int, nz: int, dz: float, delta: float, base: float, amplitude: float,
               phase: float = 0.0) -> np.ndarray:
    """Single grain under a front at base + amplitude*cos(2 pi x/nx + phase)
    (amplitude 0: flat), liquid = 1 - solid; [2, nx, ny, nz] float32."""
    x = np.arange(nx, dtype=np.float64).reshape(nx, 1, 1)
    z = np.arange(nz, dtype=np.float64).reshape(1, 1, nz)
    height = base + amplitude * np.cos(2.0 * math.pi * x / max(nx, 1) + phase)
    solid = (0.5 * (1.0 - np.tanh(np.float32(2.2 / delta) * ((z - height) * dz)))).astype(np.float32)
    phi = np.zeros((2, nx, ny, nz), np.float32)
    phi[1] = np.broadcast_to(solid, (nx, ny, nz))
    phi[0] = 1.0 - phi[1]
    return phi


def _wavy_solid(nx: int, nz: int, dz: float, delta: float, base: float, waviness: float) -> np.ndarray:
    """[nx, 1, nz] tanh solid fraction under a front at
    base + waviness*cos(2 pi x/nx)."""
    x = np.arange(nx, dtype=np.float64).reshape(nx, 1, 1)
    z = np.arange(nz, dtype=np.float64).reshape(1, 1, nz)
    h = base + waviness * np.cos(2.0 * math.pi * x / max(nx, 1))
    return (0.5 * (1.0 - np.tanh(np.float32(2.2 / delta) * ((z - h) * dz)))).astype(np.float32)


def stripe_grain_map(nx: int, ny: int, n_solid: int) -> np.ndarray:
    """[nx, ny] grain ids 1..n_solid in equal x stripes (edges at
    linspace(0, nx, n_solid+1) truncated), tests/verification_3d.py:296-301."""
    edges = np.linspace(0, nx, n_solid + 1).astype(int)
    col = np.zeros(nx, np.int32)
    for g in range(1, n_solid + 1):
        col[edges[g - 1]:edges[g]] = g
    return np.repeat(col[:, None], ny, axis=1)


def bicrystal_field(nx: int, ny: int, nz: int, dz: float, delta: float, seed_height: float,
                    split_index: int, waviness: float = 0.0, left_offset: float = 0.0,
                    right_offset: float = 0.0) -> np.ndarray:
    """phi [3, nx, ny, nz] float32: grain 1 for x < split_index, grain 2 from
    there on, each under its own (optionally wavy) front, liquid the clipped
    rest; bicrystal_phi_3d, tests/verification_3d.py:1085-1111."""
    phi = np.zeros((3, nx, ny, nz), np.float32)
    left = _wavy_solid(nx, nz, dz, delta, seed_height + left_offset, waviness)
    right = _wavy_solid(nx, nz, dz, delta, seed_height + right_offset, waviness)
    phi[1, :split_index] = np.broadcast_to(left[:split_index], (split_index, ny, nz))
    phi[2, split_index:] = np.broadcast_to(right[split_index:], (nx - split_index, ny, nz))
    phi[0] = np.clip(1.0 - phi[1] - phi[2], 0.0, 1.0)
    return phi


def alternating_multigrain_field(nx: int, ny: int, nz: int, dz: float, delta: float, seed_height: float,
                                 n_grains: int, waviness: float = 0.0) -> np.ndarray:
    """Stripes of n_grains grains under one front; with waviness the front
    is base + waviness*cos(2 pi x/nx) (alternating_multigrain_phi_3d,
    tests/verification_3d.py:1114-1135)."""
    gmap = stripe_grain_map(nx, ny, n_grains)
    phi = phi_from_grain_map_2d(gmap, n_grains, nz, dz, delta, int(seed_height))
    if waviness == 0.0:
        return phi
    solid = _wavy_solid(nx, nz, dz, delta, seed_height, waviness)
    for g in range(1, n_grains + 1):
        phi[g] = np.where((gmap == g)[:, :, None], solid, 0.0)
    phi[0] = np.clip(1.0 - phi[1:].sum(axis=0), 0.0, 1.0)
    return phi


def quaternions_of(rotations) -> np.ndarray:
    """[len+1, 4] (x, y, z, w): the liquid's identity, then one scipy Rotation
    per grain (quaternions_from_rotations, tests/verification_3d.py:304-309)."""
    q = np.zeros((len(rotations) + 1, 4), np.float64)
    q[0] = (0.0, 0.0, 0.0, 1.0)
    for g, r in enumerate(rotations, 1):
        q[g] = r.as_quat()
    return q


def orientation_library() -> dict:
    """The verification suite's named grain orientations
    (orientation_library, tests/verification_3d.py:1138-1147)."""
    from scipy.spatial.transform import Rotation
    src = np.array([[1.0, 1.0, 1.0]]) / math.sqrt(3.0)
    aligned, _ = Rotation.align_vectors(np.array([[0.0, 0.0, 1.0]]), src)
    return {"identity": Rotation.identity(),
            "y_15": Rotation.from_euler("y", 15.0, degrees=True),
            "y_30": Rotation.from_euler("y", 30.0, degrees=True),
            "y_45": Rotation.from_euler("y", 45.0, degrees=True),
            "x_30": Rotation.from_euler("x", 30.0, degrees=True),
            "tilt_xyz": Rotation.from_euler("xyz", [20.0, 35.0, 10.0], degrees=True),
            "aligned_111_to_z": aligned}
