"""Searches in one process reuse the streams, events, survivor buffers and
pinned staging of earlier ones (a per-device pool).  Their results must not
depend on what ran before: another plan, pre-verification on or off, buffers
grown past the pooled size, or buffers fixed small by RPG_SURVIVOR_CAPACITY."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CONIC = ["1", "0", "1"]  # y^2 = x^2 + 1: 440 points with |a| <= 2000, b <= 300


def expected_points(oracle):
    found = []
    o = oracle.Options(coefficients=CONIC, height=2000, first=1, last=300)
    oracle.search(o, lambda a, y, d: found.append((a, int(y), d)) or True)
    return found


def test_results_independent_of_earlier_searches(rpg, oracle, golden, monkeypatch):
    expected = expected_points(oracle)
    assert len(expected) == 440
    first, stats = rpg.point_search(CONIC, 2000, 1, 300)
    assert first == expected
    # every site of the dense curve survives: about 400,000 survivors grow
    # the buffers past the pooled size
    dense = golden["dense"]["coefficients"].split()
    a, d, s = rpg.sieve(dense, 5000, 1, 40)
    assert len(a) == s["survivor_count"] == 40 * 10001
    # buffers fixed at 1,000 survivors: the split path
    monkeypatch.setenv("RPG_SURVIVOR_CAPACITY", "1000")
    a, d, _ = rpg.sieve(dense, 5000, 1, 2)
    keys = (d.astype(np.int64) - 1) * 10001 + (a + 5000)
    assert len(a) == 20002 and len(np.unique(keys)) == 20002
    monkeypatch.delenv("RPG_SURVIVOR_CAPACITY")
    for plan, preverify in (("fast", False), ("reference", True), ("fast", True)):
        again, s = rpg.point_search(CONIC, 2000, 1, 300, plan=plan, preverify=preverify)
        assert again == expected, (plan, preverify)
        if plan == "fast":
            assert s["survivor_count"] == stats["survivor_count"]


def test_search_after_releasing_the_pool(rpg, oracle):
    expected = expected_points(oracle)
    assert rpg.point_search(CONIC, 2000, 1, 300)[0] == expected
    rpg.release_cached_resources(0)
    rpg.release_cached_resources()  # already empty
    assert rpg.point_search(CONIC, 2000, 1, 300)[0] == expected
    assert rpg.point_search(CONIC, 2000, 1, 300, plan="reference")[0] == expected
