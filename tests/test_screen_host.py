"""Host logic of the surrogate-screened scan (mpf3d.screen), no GPU: the
bounded training form of the targets, the seeded candidate sampling, and the
final answer -- the best simulated candidates -- which can only gain true
top-k members when more candidates are simulated."""
import numpy as np

from mpf3d.screen import best_simulated, bounded, sample_pairs


def test_bounded_form():
    y = np.array([[1.0, 45.0], [3.0, -90.0], [-1.0, 0.0], [0.0, 22.5]])
    b = bounded(y)
    assert np.allclose(b[:, 0], [0.0, 0.5, -1.0, -1.0])
    assert np.allclose(b[:, 1], [1.0, -2.0, 0.0, 0.5])
    r = np.linspace(0.1, 10, 50)
    assert np.all(np.diff(bounded(np.stack([r, r], 1))[:, 0]) > 0)  # monotone in the ratio


def test_sample_pairs_is_seeded_and_normalised():
    a = sample_pairs(64, seed=5)
    b = sample_pairs(64, seed=5)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    q1, q2, dT, da = a
    assert np.allclose(np.linalg.norm(q1, axis=1), 1) and np.allclose(np.linalg.norm(q2, axis=1), 1)
    assert dT.min() >= 0.25 and dT.max() <= 3.0 and da.min() >= 0.0 and da.max() <= 1.0


def test_best_simulated_ranks_by_value_and_puts_nan_last():
    known = {7: 0.5, 3: np.nan, 9: 0.9, 1: 0.1, 4: 0.7}
    assert best_simulated(known, 3).tolist() == [9, 4, 7]
    assert best_simulated(known, 5).tolist()[-1] == 3


def test_more_simulated_candidates_never_lose_true_top_members():
    rng = np.random.default_rng(0)
    truth = rng.normal(size=5000)
    k = 64
    true_top = set(np.argsort(-truth)[:k].tolist())
    known = {i: truth[i] for i in rng.choice(5000, 300, replace=False).tolist()}
    before = len(true_top & set(best_simulated(known, k).tolist()))
    for i in rng.choice(5000, 700, replace=False).tolist():
        known[i] = truth[i]
    after = len(true_top & set(best_simulated(known, k).tolist()))
    assert after >= before
    # every true top-k member that was simulated is in the answer
    assert true_top & set(known) <= set(best_simulated(known, k).tolist())
