"""Device pre-verification on the GPU: with it (the default) and without it
(RPG_SEARCH_HOST_VERIFY_ONLY / RPG_BATCH_HOST_VERIFY_ONLY) every search gives
the same points and the same modular survivor counts, while the host checks
far fewer candidates; also through the overflow paths (split pieces, batch
rerun) and for square denominators and large coefficients."""

import random

import pytest

pytestmark = pytest.mark.gpu

RECORD = "247747600 -985905640 567207969 2396040466 52485681 -470135160 82342800"


def both(rpg, coeffs, bound, first, last, **kw):
    on = rpg.point_search(coeffs, bound, first, last, **kw)
    off = rpg.point_search(coeffs, bound, first, last, preverify=False, **kw)
    return on, off


@pytest.mark.parametrize("plan", ["reference", "fast"])
@pytest.mark.parametrize("case", [
    (RECORD, 200000, 1, 20000, False),
    ("4 -37 -48 27 34 -28 49", 2000, 1, 2000, False),
    ("1 -1 0 1", 100000, 1, 300, True),
    ("-2 0 1 0 1", 3000, 3, 900, False),
], ids=["record", "c1", "square-cubic", "quartic"])
def test_single_search_same_points(rpg, plan, case):
    coeffs, bound, first, last, square = case
    (p_on, s_on), (p_off, s_off) = both(rpg, coeffs, bound, first, last, plan=plan, square=square)
    assert p_on == p_off
    assert s_on["survivor_count"] == s_off["survivor_count"]
    assert s_off["host_candidates"] == s_off["survivor_count"]
    finite = sum(1 for p in p_on if p[2] != 0)
    assert finite <= s_on["host_candidates"] <= s_on["survivor_count"]
    if plan == "reference" and s_on["survivor_count"] > 1000:
        assert s_on["host_candidates"] * 20 < s_on["survivor_count"]


def test_large_coefficients_same_points(rpg):
    rng = random.Random(5)
    for degree in (4, 7, 12):
        coeffs = [str(rng.randint(-(2 ** 160), 2 ** 160)) for _ in range(degree + 1)]
        (p_on, s_on), (p_off, s_off) = both(rpg, " ".join(coeffs), 5000, 1, 400)
        assert p_on == p_off
        assert s_on["survivor_count"] == s_off["survivor_count"]


def test_split_pieces_same_points(rpg, monkeypatch):
    # survivor buffers of 64 entries: batches arrive in many split pieces
    monkeypatch.setenv("RPG_SURVIVOR_CAPACITY", "64")
    (p_on, s_on), (p_off, s_off) = both(rpg, RECORD, 20000, 1, 300, plan="reference")
    assert p_on == p_off and p_on
    assert s_on["survivor_count"] == s_off["survivor_count"]


def batch_curves(seed, n):
    rng = random.Random(seed)
    curves = []
    for i in range(n):
        degree = rng.choice([2, 3, 4, 5, 6, 8])
        coeffs = [str(rng.randint(-200, 200)) for _ in range(degree + 1)]
        if coeffs[-1] == "0":
            coeffs[-1] = "1"
        curves.append({"coefficients": coeffs, "bound": rng.choice([300, 3000, 100000]),
                       "first": 1, "last": rng.choice([50, 500, 3000])})
    curves.append({"coefficients": RECORD.split(), "bound": 100000, "first": 1, "last": 5000})
    curves.append({"coefficients": ["1", "-1", "0", "1"], "bound": 10 ** 6, "first": 1, "last": 200,
                   "square": True})
    return curves


def test_batch_same_points_and_counts(rpg):
    curves = [c for c in batch_curves(3, 40) if rpg.is_squarefree(c["coefficients"])]
    on = rpg.batch_search(curves)
    off = rpg.batch_search(curves, preverify=False)
    assert on[0] == off[0] and on[1] == off[1]
    assert on[2] == off[2]  # per-curve modular survivors
    assert on[3]["survivors"] == off[3]["survivors"]
    assert off[3]["host_candidates"] == off[3]["survivors"]
    assert on[3]["host_candidates"] < on[3]["survivors"]
    for c, got in zip(curves[-2:], on[0][-2:]):
        assert got == rpg.point_search(c["coefficients"], c["bound"], c["first"], c["last"],
                                       square=c.get("square", False))[0]


def test_batch_rerun_same_points(rpg, monkeypatch):
    curves = [c for c in batch_curves(9, 12) if rpg.is_squarefree(c["coefficients"])]
    full = rpg.batch_search(curves)
    monkeypatch.setenv("RPG_BATCH_CAPACITY", "100")
    small = rpg.batch_search(curves)
    assert small[0] == full[0] and small[2] == full[2]
