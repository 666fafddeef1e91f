"""The failure path of the bounded mbarrier wait, without a fault: a wait on a
phase that nothing completes gives up after its poll limit, the launch
reports RPG_E_TIMEOUT through the C ABI, and the context stays usable (the
next wait, sieve and point search on it give correct results)."""

import pytest

pytestmark = pytest.mark.gpu


def test_wait_without_arrival_times_out(rpg):
    with pytest.raises(rpg.RpgError) as err:
        rpg.bounded_wait_selftest(1000, arrive=False)
    assert err.value.status == 4  # RPG_E_TIMEOUT
    assert "gave up after 1000 polls" in err.value.message


def test_wait_with_arrival_succeeds(rpg):
    rpg.bounded_wait_selftest(1000, arrive=True)
    rpg.bounded_wait_selftest(1, arrive=True)


def test_context_usable_after_timeouts(rpg, oracle):
    for _ in range(3):
        with pytest.raises(rpg.RpgError):
            rpg.bounded_wait_selftest(64, arrive=False)
    rpg.bounded_wait_selftest(64, arrive=True)
    coeffs = ["-3", "5", "-7", "11", "2"]
    points, _ = rpg.point_search(coeffs, 400, 1, 400)
    expected = []
    o = oracle.Options(coefficients=coeffs, height=400, first=1, last=400)
    oracle.search(o, lambda a, y, d: expected.append((a, int(y), d)) or True)
    assert points == expected and expected
