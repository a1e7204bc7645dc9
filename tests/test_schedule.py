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


def _round_tables(pairs, nb):
    slot, partner = [0] * nb, [0] * nb
    for k, (i, j, on) in enumerate(pairs):
        slot[i] = slot[j] = k
        partner[i], partner[j] = (j, i) if on else (-1, -1)
    return slot, partner


def _folded(w, p):
    """The sweep kernel's folded enumeration of the pairs k <= l."""
    q = p + 1
    r, c = divmod(w, q)
    if c < p - r:
        return r, r + c
    if (p & 1) and r == p // 2:
        return None
    return p - 1 - r, c - 1


def _check_overlap(nb, rounds):
    """The overlapped round of the sweep kernel: each pivot quad of round
    r+1 computes (or waits for the owner of) the super-tile of round r that
    holds its cross tile; the other warps take every super-tile the
    criticality test leaves.  Every super-tile of r must be updated exactly
    once and every next cross tile must be covered.  Returns the number of
    shared super-tiles (a quad waits on another's flag)."""
    p = nb // 2
    items = ((p + 1) // 2) * (p + 1)
    shared = 0
    for r in range(len(rounds) - 1):
        cur, nxt = rounds[r], rounds[r + 1]
        cs, _ = _round_tables(cur, nb)
        ns, npart = _round_tables(nxt, nb)
        owned, needs = {}, {}
        for kk, (x, y, on) in enumerate(nxt):
            if not on or cs[x] == cs[y]:
                continue
            k, l = cs[x], cs[y]
            ox, oy = cur[k][0] + cur[k][1] - x, cur[l][0] + cur[l][1] - y
            owner = ns[ox] if (npart[ox] == oy and min(ox, oy) < min(x, y)) else kk
            shared += owner != kk
            item = (min(k, l), max(k, l))
            needs[kk] = (item, owner)
            if owner == kk:
                assert item not in owned
                owned[item] = kk
        assert all(owned.get(item) == owner for item, owner in needs.values())
        done = set(owned)
        for w in range(items):
            f = _folded(w, p)
            if f is None or f[0] == f[1]:
                continue
            k, l = f
            p1, p2 = npart[cur[k][0]], npart[cur[k][1]]
            critical = (p1 >= 0 and cs[p1] == l) or (p2 >= 0 and cs[p2] == l)
            assert critical == (f in owned)
            if not critical:
                assert f not in done
                done.add(f)
        assert done == {(k, l) for k in range(p) for l in range(k + 1, p)}
    return shared


@pytest.mark.parametrize("nb", [2, 4, 6, 10, 16, 40, 64, 82, 128])
def test_overlapped_round_covers_every_super_tile_round_robin(nb):
    rounds = [[(*sorted(_rr_pair(k, r, nb)), True) for k in range(nb // 2)] for r in range(nb - 1)]
    _check_overlap(nb, rounds)


@pytest.mark.parametrize("nb", [66, 82, 98, 114, 128])
def test_overlapped_round_covers_every_super_tile_two_level(nb):
    table = O.two_level_schedule(nb).reshape(-1, 2)
    p = nb // 2
    rounds = [[(int(i), int(j) if j >= 0 else -1 - int(j), bool(j >= 0)) for i, j in table[r * p:(r + 1) * p]]
              for r in range(len(table) // p)]
    assert _check_overlap(nb, rounds) > 0   # shared super-tiles occur: the flag path is exercised


# ---- routing between the batched and the grid kernels (host side) ---------

def test_routing_cost_model(msq):
    """FP32 mode: the cost model moves the largest matrices to the grid
    kernels only where their one-CTA solves would outlast the batch (GB300
    timings: a lone n = 512 solves in 17.6 ms on the grid kernels against
    52 ms on one CTA; eight n = 384 take 76 ms on the grid kernels one after
    another against 20 ms batched)."""
    route = lambda orders, mode=0: msq.jacobi_route(orders, mode).tolist()
    assert route([300]) == [1]                       # lone: grid
    assert route([300] * 9) == [0] * 9               # nine concurrent CTAs win
    assert route([384] * 8) == [0] * 8
    assert route([512, 512]) == [1, 1]
    assert route([512] * 4) == [0] * 4
    assert route([256]) == [0]                       # up to 256: always batched
    assert route([2048, 64, 100]) == [1, 0, 0]       # above 1024: always grid
    # a fallback-sized mix: only its largest member outlasts the rest
    mix = [367, 230, 32, 399, 45, 83, 45, 125, 176, 275, 252, 330, 81, 300, 344,
           153, 127, 36, 387, 154, 143, 119, 404, 387, 378, 105, 154, 510]
    assert [n for n, g in zip(mix, route(mix)) if g] == [510]
    # a throughput-bound batch stays on the batched kernels
    rng = np.random.default_rng(0)
    big = np.floor(np.exp(rng.uniform(np.log(16), np.log(513), 4096))).astype(int)
    assert sum(route(big)) == 0


def test_routing_two_level_modes(msq):
    """The two-level modes keep the rule they were built with: a matrix
    above 256 goes to the grid kernels when at most eight are in the batch."""
    for mode in (1, 2, 3):
        assert msq.jacobi_route([300] * 8, mode).tolist() == [1] * 8
        assert msq.jacobi_route([300] * 9, mode).tolist() == [0] * 9
        assert msq.jacobi_route([2048, 300] + [400] * 9, mode).tolist() == [1] + [0] * 10
    with pytest.raises(Exception):
        msq.jacobi_route([300], 4)
