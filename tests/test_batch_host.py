"""Host-side checks of the batch and serving ABI that need no GPU: argument
validation happens before any device work, and the seeded workloads are
reproducible with the distributions they document."""

import ctypes
import math

import pytest


def test_batch_search_rejects_bad_arguments(rpg):
    lib = rpg.load()
    stats = rpg.BatchStats()
    cb = rpg.BATCH_POINT_CB(lambda *a: 1)
    status = lib.rpg_batch_search(None, -1, -1, 0, cb, None, None, None, ctypes.byref(stats))
    assert status == 1 and b"must not be NULL" in lib.rpg_last_error()
    status = lib.rpg_batch_search(None, 0, -1, 0, rpg.BATCH_POINT_CB(), None, None, None, None)
    assert status == 1


def test_server_rejects_bad_options(rpg):
    lib = rpg.load()
    handle = ctypes.c_void_p()
    for lanes, budget, batch in ((0, 1 << 30, 16), (17, 1 << 30, 16), (2, 0, 16), (2, 1 << 30, 0)):
        opts = rpg.ServerOptions(-1, lanes, budget, batch)
        assert lib.rpg_server_create(ctypes.byref(opts), ctypes.byref(handle)) == 1
    assert lib.rpg_server_create(None, ctypes.byref(handle)) == 1


def test_server_wait_rejects_null_handle(rpg):
    lib = rpg.load()
    done = ctypes.c_int32(7)
    assert lib.rpg_server_wait(None, 1, 0.0, rpg.POINT_CB(), None, ctypes.byref(done), None) == 1


def test_mixed_batch_is_seeded_and_in_range(rpg):
    import workloads

    a = workloads.mixed_batch(64)
    b = workloads.mixed_batch(64)
    assert a == b
    for c in a:
        degree = len(c["coefficients"]) - 1
        assert degree in (3, 4, 5, 6, 8, 10)
        for x in c["coefficients"]:
            assert 8 <= abs(int(x)).bit_length() <= 64
        assert 10**3 <= c["bound"] <= 10**6 and 10**3 <= c["last"] <= 10**6
        assert rpg.is_squarefree(c["coefficients"])
    # log-uniform: about half the heights below sqrt(1e3 * 1e6)
    below = sum(c["bound"] < math.sqrt(1e9) for c in workloads.mixed_batch(400))
    assert 140 < below < 260


def test_other_workloads_match_their_definitions(rpg):
    import workloads

    for c in workloads.wide_degree(8):
        assert 12 <= len(c["coefficients"]) - 1 <= 40
        assert all(100 <= abs(int(x)).bit_length() <= 256 for x in c["coefficients"])
        assert c["bound"] == c["last"] == 10**5 and len(c["intervals"]) == 3
    for c in workloads.square_cubics(8):
        beta, alpha, zero, one = map(int, c["coefficients"])
        assert zero == 0 and one == 1 and abs(alpha) <= 10**12 and abs(beta) <= 10**12
        assert c["square"] and c["last"] == 46340 and c["bound"] == 10**9
    stream = workloads.serving_stream(300)
    times = [t for t, _, _ in stream]
    assert times == sorted(times)
    assert 0.8 < len(stream) / times[-1] / 200.0 < 1.25  # about 200 arrivals per second
    first = sum(f for _, _, f in stream) / len(stream)
    assert 0.2 < first < 0.4
    for _, req, _ in stream:
        assert 2 <= len(req["coefficients"]) - 1 <= 12
        assert 10**2 <= req["bound"] <= 10**6 and req["last"] == req["bound"]


def test_reduced_site_count_matches_a_direct_count(rpg):
    import workloads

    mu = workloads.mobius(60)
    for h, first, last in ((7, 1, 30), (20, 5, 60), (1, 1, 1)):
        direct = sum(1 for d in range(first, last + 1) for a in range(-h, h + 1)
                     if math.gcd(a, d) == 1)
        assert workloads.reduced_sites(h, first, last, mu) == direct
