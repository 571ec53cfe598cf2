"""The learned proposal's prefix rules on the host (no GPU): the top-score margin a
graph needs is exact (it holds the needed prefix, and one proposal fewer does not),
and the calibrated margin for unseen graphs covers every training graph's need."""
import numpy as np

from minimumcyclebasis_gb300.learned import calibrate_margin, needed_margin, proposal_prefix, tail_prefix


def test_needed_margin_is_the_smallest_that_holds():
    rng = np.random.default_rng(0)
    for _ in range(300):
        K = int(rng.integers(5, 400))
        N = int(rng.integers(1, K))
        w = np.sort(rng.integers(1, 25, K)).astype(np.int32)  # ties in weight, as in rank order
        logits = rng.normal(size=K).astype(np.float32)
        K_needed = int(rng.integers(1, K + 1))
        m = needed_margin(logits, w, N, K_needed)
        k, U = proposal_prefix(logits, w, N, m)
        assert k >= K_needed and U >= w[K_needed - 1]
        if m > 0:
            k2, _ = proposal_prefix(logits, w, N, m - 1.0 / N)
            assert k2 < K_needed


def test_calibrated_margin_covers_the_training_needs():
    needs = [0.12, 0.4, 0.07]
    m = calibrate_margin(needs)
    assert m >= max(needs) and m == max(needs) * 1.25 + 0.05
    assert calibrate_margin([]) == 0.05


def test_tail_rule_keeps_whole_weight_classes():
    rng = np.random.default_rng(3)
    w = np.sort(rng.integers(1, 10, 500)).astype(np.int32)
    logits = rng.normal(size=500).astype(np.float32)
    for eps in (3.0, 1.0, 0.1):
        k, U = tail_prefix(logits, w, 5.0, eps)
        assert k == len(w) or w[k] > U  # the prefix ends at the end of U's weight class
        assert (w[:k] <= U).all()
