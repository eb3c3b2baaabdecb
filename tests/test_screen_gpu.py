"""Surrogate-screened scan on the GPU at a reduced scale (4096 candidate grain
pairs): against an exhaustive simulation of every candidate, the surrogate's
top-64 must be far better than the same simulation budget spent on random
candidates (the method without the network), and cheaper than the exhaustive
scan; a refit round re-ranks every simulated candidate by its simulated value
and can only add true top-k members."""
import pytest

pytestmark = pytest.mark.gpu
pytest.importorskip("torch")


def test_screening_beats_random_picks_of_the_same_budget():
    from mpf3d.screen import screen
    rep = screen(n_candidates=4096, n_train=512, top_k=64, n_audit=64, epochs=300, exhaustive=True, seed=3,
                 rounds=2, recheck=256)
    ex = rep["exhaustive"]
    # the refinement round re-ranks a superset of the checked top by simulated values
    assert ex["final_top_k_overlap"] >= ex["top_k_overlap"], rep
    assert rep["final"]["simulated"] > 512 + 64 + 64, rep
    gain = rep["objective_mean_top_simulated"] - rep["objective_mean_random_simulated"]
    achievable = ex["true_top_mean"] - rep["objective_mean_random_simulated"]
    assert gain > 0.5 * achievable, rep
    assert ex["top_k_overlap"] >= 10 * 64 / 4096, rep
    assert rep["surrogate_error_audit"]["corr"][0] > 0.7, rep
    assert ex["gpu_seconds"] > rep["gpu_seconds"]["screened_total"]
