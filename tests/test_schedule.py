"""The two-level Jacobi pairing (host side, no GPU): the library's table
equals the oracle's restatement for every block count up to 256, each round
is a perfect matching of the blocks, every block pair rotates exactly once
per sweep, and each stage's rotations stay inside the stage's 64-index
super-pairs (the property that makes their product block diagonal)."""
import numpy as np
import pytest

import oracle as O


def _rr_pair(pair, rnd, m):
    def slot(s):
        return 0 if s == 0 else 1 + (s - 1 - rnd % (m - 1)) % (m - 1)
    a, b = slot(pair), slot(m - 1 - pair)
    return min(a, b), max(a, b)


@pytest.mark.parametrize("blocks", list(range(2, 258, 2)))
def test_library_table_equals_oracle(msq, blocks):
    assert np.array_equal(msq.jacobi_schedule(blocks), O.two_level_schedule(blocks))


@pytest.mark.parametrize("blocks", [2, 8, 16, 18, 66, 84, 96, 100, 116, 128])
def test_matching_coverage_and_stage_locality(blocks):
    table = O.two_level_schedule(blocks)
    supers = (blocks + 7) // 8
    supers += supers % 2
    assert table.shape == (7 + 8 * (supers - 1), blocks // 2, 2)
    seen = set()
    for r, rnd in enumerate(table):
        stage = 0 if r < 15 else (r - 7) // 8
        groups = {}
        for x in range(supers // 2):
            p, q = _rr_pair(x, stage, supers)
            groups[p] = groups[q] = x
        used = set()
        for i, j in rnd:
            active = j >= 0
            j = j if active else -1 - j
            assert i < j and i not in used and j not in used
            used |= {i, j}
            if active:
                assert (i, j) not in seen
                seen.add((i, j))
                assert groups[i // 8] == groups[j // 8]
        assert used == set(range(blocks))
    assert len(seen) == blocks * (blocks - 1) // 2


def test_schedule_rejects_bad_block_counts(msq):
    for blocks in (0, 1, 3, -2):
        with pytest.raises(msq.MsqError):
            msq.jacobi_schedule(blocks)


def test_two_level_oracle_converges_like_round_robin():
    """The oracle's blocked Jacobi in the two-level order reaches the same
    tolerance within one sweep of the round-robin order."""
    for n, seed in ((300, 1), (400, 2), (512, 3)):
        a = O.wishart(n, seed)
        _, _, rr, _ = O.jacobi_blocked(a, 1e-4, 15)
        w, v, tl, ratio = O.jacobi_blocked(a, 1e-4, 15, two_level=True)
        assert ratio <= 1e-4 and abs(tl - rr) <= 1
        lam = np.linalg.eigvalsh(a)
        assert np.abs(np.sort(w) - lam).max() <= 3 * n * 2.0 ** -24 * lam.max()
