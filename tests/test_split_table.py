"""The grouped-contraction planner's split of a table above the library's
slot and entry limits (engine._split_table): host logic, no GPU."""
import random

import pytest

from carcassonne_gb300.engine import _split_table


def _check(n_c, entries, limit, max_entries):
    calls = _split_table(n_c, entries, limit, max_entries)
    seen = {c: [] for c in range(n_c)}
    first = {}
    for a_idx, b_idx, c_idx, ents, acc in calls:
        assert 1 <= len(c_idx) <= limit and len(a_idx) <= limit and len(b_idx) <= limit
        assert len(ents) <= max_entries
        assert len(set(c_idx)) == len(c_idx)
        if acc:
            assert len(c_idx) == 1 and c_idx[0] in first  # a later part of one output
        for c in c_idx:
            if not acc:
                assert c not in first  # written by exactly one non-accumulating call
                first[c] = True
        for a, b, c in ents:
            assert 0 <= a < len(a_idx) and 0 <= b < len(b_idx) and 0 <= c < len(c_idx)
            seen[c_idx[c]].append((a_idx[a], b_idx[b]))
    assert sorted(first) == list(range(n_c))  # every output written, including those with no entry
    for c in range(n_c):
        assert seen[c] == [(a, b) for a, b, cc in entries if cc == c]  # each output's order kept
    return calls


@pytest.mark.parametrize("seed", range(8))
def test_split_random_tables(seed):
    rng = random.Random(seed)
    n_c = rng.randint(1, 150)
    n_a, n_b = rng.randint(1, 120), rng.randint(1, 120)
    entries = [(rng.randrange(n_a), rng.randrange(n_b), rng.randrange(n_c)) for _ in range(rng.randint(0, 1500))]
    _check(n_c, entries, 64, 512)


def test_split_output_needing_more_than_the_limit():
    # one output fed by 150 distinct A operands: three parts, the later two accumulating
    entries = [(i, i % 7, 1) for i in range(150)] + [(3, 2, 0), (5, 1, 2)]
    calls = _check(3, entries, 64, 512)
    parts = [c for c in calls if c[2] == [1]]
    assert len(parts) == 3 and [p[4] for p in parts] == [False, True, True]


def test_split_small_table_is_one_call():
    entries = [(0, 0, 0), (1, 0, 1), (0, 1, 1)]
    calls = _check(2, entries, 64, 512)
    assert len(calls) == 1 and calls[0][3] == entries
