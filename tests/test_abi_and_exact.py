"""CPU-only checks of librpgpu: it loads, exports every declared C-ABI symbol,
and its exact arithmetic and CLI parsing agree with the oracle.  No call here
reaches a CUDA kernel."""

import ctypes
import random

import pytest


def test_library_exports_every_declared_function(rpg):
    lib = rpg.load()
    names = rpg.declared_functions()
    assert len(names) >= 11
    for name in names:
        assert hasattr(lib, name), name
    assert lib.rpg_abi_version() == 3


def test_header_declares_the_sieve_boundary(rpg):
    names = set(rpg.declared_functions())
    assert {"rpg_sieve_run", "rpg_point_search", "rpg_is_squarefree", "rpg_square_root",
            "rpg_cli_main", "rpg_last_error"} <= names


def _random_poly(rng, degree, bits):
    coeffs = [rng.randint(-(2**bits), 2**bits) for _ in range(degree + 1)]
    if coeffs[-1] == 0:
        coeffs[-1] = 1
    return coeffs


def test_squarefree_agrees_with_oracle(rpg, oracle):
    rng = random.Random(3)
    for _ in range(60):
        degree = rng.randint(1, 9)
        coeffs = _random_poly(rng, degree, rng.choice([3, 20, 80]))
        assert rpg.is_squarefree(coeffs) == oracle.is_squarefree(coeffs), coeffs


def _polymul(p, q):
    out = [0] * (len(p) + len(q) - 1)
    for i, a in enumerate(p):
        for j, b in enumerate(q):
            out[i + j] += a * b
    return out


def test_non_squarefree_detected(rpg, oracle):
    rng = random.Random(5)
    for _ in range(25):
        g = _random_poly(rng, rng.randint(1, 3), 30)
        h = _random_poly(rng, rng.randint(0, 4), 30)
        f = _polymul(_polymul(g, g), h)
        assert not rpg.is_squarefree(f)
        assert not oracle.is_squarefree(f)
    assert not rpg.is_squarefree([1, -2, 1])
    assert rpg.is_squarefree([1] + [0] * 99 + [1])


def test_square_root_agrees_with_oracle(rpg, oracle):
    rng = random.Random(9)
    curves = [[rng.randint(-50, 50) for _ in range(7)] for _ in range(4)]
    curves += [_random_poly(rng, 12, 200), _random_poly(rng, 5, 64), [0, 0, 0, 1, 0, 1]]
    curves = [c if c[-1] else c[:-1] + [1] for c in curves]
    for coeffs in curves:
        for _ in range(150):
            a = rng.randint(-10**6, 10**6)
            b = rng.randint(0, 10**6)
            assert rpg.square_root(coeffs, a, b) == oracle.square_root(coeffs, a, b)


def test_square_root_finds_constructed_points(rpg, oracle):
    # f = y0^2 - x^2 h(x) style curves: (a, b) = (0, 1) is a point with y = y0
    rng = random.Random(13)
    for _ in range(30):
        y0 = rng.randint(1, 10**30)
        coeffs = [y0 * y0] + [rng.randint(-10**20, 10**20) for _ in range(rng.randint(2, 8))]
        if coeffs[-1] == 0:
            coeffs[-1] = 7
        assert rpg.square_root(coeffs, 0, 1) == y0
        # infinity: even degree with square leading coefficient
        lead = rng.randint(1, 10**25)
        even = coeffs[:1] + [3] * (2 * rng.randint(1, 4) - 1) + [lead * lead]
        assert rpg.square_root(even, 1, 0) == lead
        odd = coeffs[:1] + [3] * (2 * rng.randint(1, 4)) + [5]
        assert rpg.square_root(odd, 1, 0) == 0


def test_large_values_square_root(rpg, oracle):
    rng = random.Random(17)
    for bits in (70, 127, 128, 129, 200, 1000, 4000):
        for _ in range(10):
            y = rng.getrandbits(bits) | 1
            for value in (y * y, y * y + 1, y * y - 1):
                # constant polynomial of degree 1 with zero slope is not allowed; use
                # f(x) = value + x^2 at (0, 1).
                coeffs = [value, 0, 1]
                expected = oracle.square_root(coeffs, 0, 1)
                assert rpg.square_root(coeffs, 0, 1) == expected


BAD_ARGS = [
    ["1 0 1"], ["1 0 1", "0"], ["1 0 1", "abc"], ["1 0 1", "5x"], ["1 0 1", "99999999999999999999"],
    ["1 0 1", "4611686018427387904"], ["1 0 1", "5", "-x"], ["1 0 1", "5", "-dl"],
    ["1 0 1", "5", "-dl", "0"], ["1 0 1", "5", "-du", "2147483648"], ["1 0 1", "5", "-dl", "6"],
    ["1 0 1", "5", "-l", "1", "-l", "2"], ["1 0 1", "5", "-l", "2", "-u", "1"],
    ["1 0 1", "5", "-l", "0", "-u", "1", "-l", "0.5", "-u", "2"], ["1 0 1", "5", "-u", "1", "-u", "2"],
    ["1 0 1", "5", "-l", "1e10001"], ["1 0 1", "5", "-l", "x"], ["1 0 1", "5", "--batch-size", "0"],
    ["1 0 1", "5", "--batch-size", "65537"], ["1 0 1", "5", "--batch-size", "abc"],
    ["1 0 1", "5", "--batch-size"], ["1 0 1", "5", "--devices", ""], ["1 0 1", "5", "--devices", ","],
    ["1 0 1", "5", "--devices", "0,"], ["1 0 1", "5", "--devices", "0,0"],
    ["1 0 1", "5", "--devices", "-1"], ["1 0 1", "5", "--devices", "+0"],
    ["1 0 1", "5", "--devices", "99999999999999999999999"], ["1 0 1", "5", "--devices"],
    ["1", "5"], ["1 x 1", "5"], ["1 0 0", "5"], ["1 " + "0 " * 100 + "1", "5"], ["1 -2 1", "5"],
    ["1 0 1", "5", "--devices", ",0"], ["1 0 1", "5", "--devices", "0,,1"],
    ["1 0 1", "5", "--devices", "1,1,x"], ["1 0 1", "5", "--devices", "0a"],
    ["1 0 1", "5", "--devices", "2147483648"], ["1 0 1", "5", "--devices", "0,x,"],
    ["1 0 1", "5", "-l", ".e99999"], ["1 0 1", "5", "-l", "1e"], ["1 0 1", "5", "-l", "1e+"],
    ["1 0 1", "5", "-l", "--"], ["1 0 1", "5", "-u", "."], ["1 0 1", "5", "-l", "e5"],
    ["1 0 1", "5", "-l", "1.5.3"], ["1 0 1", "5", "-l", "1", "-u", "0.5e0"],
    ["1 0 1", "5", "-l", "1e99999x"], ["1 0 1", "5", "-l", "1", "-l"], ["1 0 1", "5", "-l"],
    ["1 0 1", "5", "-f"], ["1 0 1", "5 "], ["+ 1", "5"], ["1 0 -0", "5"], ["1 0 +00", "5"],
    ["1 0 1", "5", "-dl", "3", "-du", "2"], ["1 0 1", "5", "--square-denominators", "-dl", "46341"],
    ["1 0 1", "5", "-l", "-1", "-u", "1e4", "-u", "2e4"],
]


@pytest.mark.parametrize("args", BAD_ARGS, ids=[" ".join(a)[:40] for a in BAD_ARGS])
def test_cli_rejects_like_the_reference(rpg, oracle, args):
    """Invalid command lines exit 1 with the reference's message and no stdout."""
    result = rpg.cli(args)
    code, out, err, _ = oracle.run(["ratpoints_gpu", *args])
    assert result.returncode == 1 and result.stdout == b""
    assert code == 1
    assert result.stderr.decode().strip() == err


def test_cli_help(rpg):
    result = rpg.cli(["--help"])
    assert result.returncode == 0 and b"Usage: ratpoints_gpu" in result.stdout
    assert rpg.cli([]).returncode == 1


def test_bounded_wait_selftest_rejects_bad_polls(rpg):
    # argument checks come before any CUDA call
    for polls in (0, -5, (1 << 20) + 1):
        with pytest.raises(rpg.RpgError) as err:
            rpg.bounded_wait_selftest(polls, arrive=True)
        assert err.value.status == 1


def test_release_cached_resources_without_searches(rpg):
    # nothing pooled yet in this process: no CUDA call is made
    rpg.release_cached_resources()
    rpg.release_cached_resources(0)
