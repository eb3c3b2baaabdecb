"""Host input restatements against the inputs recorded in the golden files
(which the reference's own host helpers produced)."""
import numpy as np
import pytest

from mpf3d import inputs
from _helpers import golden_files, golden_id

SC = ["dx", "dt", "T_melt", "Sf", "eps0_sl", "w0_sl", "a0", "delta_a", "mu_a", "p_round",
      "g2_floor", "ksi", "theta_c_rad"]


@pytest.mark.parametrize("path", golden_files("run"), ids=golden_id)
def test_interaction_matrices_and_normals(path):
    g = np.load(path)
    N = g["phi0"].shape[0]
    vals = dict(zip(SC, g["scalars"]))
    phys = inputs.Physics(delta_a=float(vals["delta_a"]), p_round=float(vals["p_round"]),
                          ksi=float(vals["ksi"]))
    wij, aij, mij = inputs.matrices_for(phys, N)
    assert np.array_equal(wij, g["wij"]) and np.array_equal(aij, g["aij"]) and np.array_equal(mij, g["mij"])
    n111 = inputs.rotated_n111(g["quats"])
    assert np.abs(n111 - g["n111"]).max() <= 2e-7
    d = phys.derived()
    assert d["eps0_sl"] == float(vals["eps0_sl"]) and d["w0_sl"] == float(vals["w0_sl"])
    assert d["g2_floor"] == float(vals["g2_floor"])


def test_random_quaternions_match_reference_draws():
    g = np.load(golden_files("run")[0])
    for p in golden_files("run"):
        g = np.load(p)
        if "voronoi" in p:
            q = inputs.random_quaternions(g["quats"].shape[0] - 1, 23)
            assert np.array_equal(q, g["quats"])
            return
    pytest.skip("no voronoi golden")


def test_voronoi_case_is_a_partition():
    c = inputs.voronoi_case(16, 12, 20, 5, 6, seed=1)
    s = c.phi.astype(np.float64).sum(axis=0)
    assert np.abs(s - 1.0).max() < 1e-6
    assert c.phi.min() >= 0.0 and c.phi.max() <= 1.0
    assert c.n111.shape == (6, 8, 3) and c.wij.shape == (6, 6)
