"""Serving loop: every answer equals the single search of the same request
(all points, or the first point for first-point requests), whether the
request runs alone or in a mix arriving over time; errors stay per request."""

import random
import threading
import time

import pytest

pytestmark = pytest.mark.gpu


def single(rpg, c, first_only=False):
    points, _ = rpg.point_search(c["coefficients"], c["bound"], c["first"], c["last"],
                                 intervals=c.get("intervals", ()),
                                 include_infinity=c.get("include_infinity", True),
                                 square=c.get("square", False),
                                 stop_after=1 if first_only else None)
    return points


def requests(rpg, rng, n):
    out = []
    while len(out) < n:
        degree = rng.randint(2, 12)
        coeffs = [str(rng.choice((-1, 1)) * rng.getrandbits(rng.randint(4, 40))) for _ in range(degree + 1)]
        if coeffs[-1] == "0" or not rpg.is_squarefree(coeffs):
            continue
        h = int(10 ** rng.uniform(2, 4.5))
        c = {"coefficients": coeffs, "bound": h, "first": 1, "last": min(h, 3000)}
        if rng.random() < 0.2:
            lo = rng.uniform(-3, 3)
            c["intervals"] = [(f"{lo:.3f}", f"{lo + 1:.3f}")]
        out.append((c, rng.random() < 0.3))
    return out


def test_answers_equal_single_searches(rpg, golden):
    dense = golden["dense"]["coefficients"].split()
    rng = random.Random(8)
    reqs = requests(rpg, rng, 40)
    reqs += [({"coefficients": dense, "bound": 3000, "first": 1, "last": 300}, False),
             ({"coefficients": dense, "bound": 3000, "first": 1, "last": 300}, True),
             ({"coefficients": dense, "bound": 150000, "first": 1, "last": 20}, True),
             ({"coefficients": ["17", "0", "0", "1"], "bound": 5000, "first": 1, "last": 900,
               "include_infinity": False}, True)]
    with rpg.Server(lanes=3) as server:
        ids = [server.submit(c, first) for c, first in reqs]
        for rid, (c, first) in zip(ids, reqs):
            status, points, stats = server.wait(rid)
            assert status == 0
            assert points == single(rpg, c, first), (c, first)
            assert stats["latency_ms"] >= stats["queue_ms"] >= 0
            assert stats["waves"] >= (0 if first else 1)


def test_alone_and_in_a_poisson_mix(rpg):
    """Requests arriving over time (exponential gaps, mean 5 ms) give the same
    answers as the same requests submitted one at a time to an idle server."""
    rng = random.Random(21)
    reqs = requests(rpg, rng, 60)
    with rpg.Server(lanes=2) as server:
        alone = []
        for c, first in reqs[:12]:
            rid = server.submit(c, first)
            alone.append(server.wait(rid)[1])
        ids = [None] * len(reqs)

        def feed():
            for i, (c, first) in enumerate(reqs):
                time.sleep(rng.expovariate(200.0))
                ids[i] = server.submit(c, first)

        t = threading.Thread(target=feed)
        t.start()
        t.join()
        mixed = [server.wait(rid) for rid in ids]
    for (c, first), (status, points, _) in zip(reqs, mixed):
        assert status == 0
        assert points == single(rpg, c, first)
    assert [m[1] for m in mixed[:12]] == alone


def test_errors_stay_with_their_request(rpg, golden):
    dense = golden["dense"]["coefficients"].split()
    with rpg.Server(lanes=1) as server:
        good = server.submit({"coefficients": dense, "bound": 500, "first": 1, "last": 40})
        bad = server.submit({"coefficients": ["1", "2", "1"], "bound": 100, "first": 1, "last": 9})
        bad_first = server.submit({"coefficients": ["1", "2", "1"], "bound": 100, "first": 1,
                                   "last": 9}, True)
        with pytest.raises(rpg.RpgError):
            server.submit({"coefficients": ["1", "q"], "bound": 100, "first": 1, "last": 9})
        assert server.wait(bad)[0] == 6
        assert server.wait(bad_first)[0] == 6
        status, points, _ = server.wait(good)
        assert status == 0 and points == single(rpg, {"coefficients": dense, "bound": 500,
                                                      "first": 1, "last": 40})


def test_first_point_at_infinity_needs_no_device_work(rpg):
    with rpg.Server(lanes=1) as server:
        rid = server.submit({"coefficients": ["5", "0", "0", "1"], "bound": 10**6, "first": 1,
                             "last": 10**6}, True)
        status, points, stats = server.wait(rid)
    assert status == 0 and points == [(1, 0, 0)] and stats["waves"] == 0


def test_wait_timeout(rpg, golden):
    dense = golden["dense"]["coefficients"].split()
    with rpg.Server(lanes=1) as server:
        rid = server.submit({"coefficients": dense, "bound": 400000, "first": 1, "last": 3000})
        first = server.wait(rid, timeout_ms=0.0)
        final = first if first is not None else server.wait(rid)
        assert final[0] == 0
