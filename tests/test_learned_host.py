"""Host-side pieces of the learned proposal that need no GPU."""
import numpy as np
import pytest

from aquagpusph_gb300 import learned as Lm


def test_pair_ring_keeps_the_newest_pairs():
    ring = Lm.PairRing(3)
    for k in range(7):
        ring.push(k)
    assert len(ring) == 3 and ring.pushed == 7
    assert sorted(ring.items) == [4, 5, 6]
    rng = np.random.default_rng(0)
    assert {ring.sample(rng) for _ in range(50)} == {4, 5, 6}


def test_pair_ring_rejects_zero_capacity():
    with pytest.raises(ValueError):
        Lm.PairRing(0)
