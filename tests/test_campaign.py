"""Campaign helper: many curves in one batched call, answers in the form the
reference's per-curve command-line callers read (rank31_family_hunt.py)."""

import random

import pytest


def _points_of(stdout):
    seen, points = set(), []
    for line in stdout.splitlines():
        a, y, b = (int(v) for v in line.strip("()").split(" : "))
        key = (a, abs(y), b)
        if key not in seen:
            seen.add(key)
            points.append(key)
    return points


def test_format_points_matches_cli_output(golden):
    import campaign
    for case in golden["oracle_cases"]:
        points = _points_of(case["stdout"])
        assert campaign.format_points(points, include_infinity=True) == case["stdout"]


@pytest.mark.gpu
def test_search_many_matches_command_line(rpg):
    import campaign
    rng = random.Random(31)
    requests = []
    while len(requests) < 12:
        alpha, beta = rng.randint(-300, 300), rng.randint(-300, 300)
        coeffs = [beta, alpha, 0, 1]
        if 4 * alpha ** 3 + 27 * beta ** 2 == 0:
            continue
        requests.append({"coefficients": coeffs, "height": rng.choice([2000, 20000, 200000]),
                         "dl": 1, "du": rng.choice([300, 3000])})
    results, _ = campaign.search_many(requests)
    for r, got in zip(requests, results):
        assert got["status"] == 0
        cli = rpg.cli([" ".join(map(str, r["coefficients"])), r["height"], "-dl", r["dl"], "-du", r["du"],
                       "--batch-size", "65536", "-i", "-v"])
        assert cli.returncode == 0
        assert got["stdout"] == cli.stdout.decode()
        assert got["exact_survivors"] == rpg.parse_metrics(cli.stderr)["exact_survivors"]
