"""ratpoints_gpu command line on the GPU: byte-exact stdout against the
reference's own oracle outputs and known answers, and the option semantics
against the oracle's restatement of the reference CLI."""

import hashlib
from fractions import Fraction

import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("plan", ["reference", "fast"])
def test_reference_oracle_cases(rpg, golden, plan):
    # tests/test_multi_gpu.py:77-93 (with --batch-size 3) and compare_with_ratpoints.py cases
    for case in golden["oracle_cases"]:
        common = [case["coefficients"], case["height"], "-dl", case["first"], "-du", case["last"]]
        for extra in ([], ["--batch-size", "3"]):
            result = rpg.cli([*common, *extra, "--sieve-plan", plan, "-v"])
            assert result.returncode == 0, result.stderr
            assert result.stdout.decode() == case["stdout"], (case["coefficients"], extra)
            metrics = rpg.parse_metrics(result.stderr)
            assert metrics["denominators"] == min(case["last"], case["height"]) - case["first"] + 1


OPTIONS = [[], ["-i"], ["-y"], ["-z"], ["-1"], ["-i", "-1"],
           ["-l", "-1", "-u", "0", "-l", "0.5", "-u", "2"], ["-i", "-1", "-l", "1", "-u", "2"],
           ["-f", "%x,%y,%z", "-fs", "[", "-fm", ";", "-fe", "]"], ["-f", "--devices"],
           ["-i", "-I", "-y", "-Y"], ["-z", "-fs", "S", "-fe", "E\\n"], ["-y", "-f", "%x %y %q %%\\%\\t|"],
           ["-l", "-3/2"][:0] + ["-u", "-0.5"], ["-l", "0.25"], ["-s", "-k", "-K", "-j", "-J", "-q"],
           ["-Z", "-z", "-1"], ["-fm", "\\n--\\n", "-i"],
           ["-f", "%\\%x%", "-fs", "\\%a\\q\\", "-fe", "%"], ["-y", "-f", "%y%x\\\\%z\\"]]


@pytest.mark.parametrize("option", OPTIONS, ids=[" ".join(o) or "default" for o in OPTIONS])
def test_option_matrix(rpg, oracle, option):
    # tests/test_multi_gpu.py:95-108 on "1 0 1" 40 -du 23 --batch-size 4
    command = ["1 0 1", "40", "-du", "23", "--batch-size", "4", *option]
    code, expected, _, _ = oracle.run(["ratpoints_gpu", *command])
    assert code == 0
    result = rpg.cli(command)
    assert result.returncode == 0, result.stderr
    assert result.stdout == expected
    if option[:1] == ["-1"] or option[:2] == ["-i", "-1"]:
        assert len(expected.splitlines()) == 1


def test_stop_after_first_metrics(rpg, oracle):
    # -1 stops after the batch holding the first accepted point
    command = ["1 0 1", "40", "-du", "23", "--batch-size", "4", "-i", "-1", "-l", "1", "-u", "2",
               "-v"]
    code, expected, _, metrics = oracle.run(["ratpoints_gpu", *command])
    assert code == 0 and expected
    result = rpg.cli([*command, "--sieve-plan", "reference"])
    assert result.stdout == expected
    got = rpg.parse_metrics(result.stderr)
    for key in ("denominators", "survivors", "exact_survivors", "words"):
        assert got[key] == metrics[key], key


def test_dense_known_answer(rpg, golden):
    # tests/test_multi_gpu.py:122-130 and compare_with_ratpoints.py:78-89
    dense = golden["dense"]
    result = rpg.cli([dense["coefficients"], "5000", "-du", "2", "-v", "--sieve-plan", "reference"])
    assert result.returncode == 0
    assert result.stdout.decode() == dense["stdout"]
    assert b"survivors=20002 exact_survivors=1" in result.stderr
    fast = rpg.cli([dense["coefficients"], "5000", "-du", "2", "-z", "-v"])
    assert fast.returncode == 0 and b"exact_survivors=1" in fast.stderr


def test_square_denominator_known_answer(rpg, golden):
    kat = golden["square_kat"]
    for plan in ("reference", "fast"):
        result = rpg.cli([*kat["args"], "--sieve-plan", plan])
        assert result.returncode == 0
        assert kat["contains"] in result.stdout.decode().splitlines()


def test_square_denominators_match_oracle(rpg, oracle):
    for command in (["1 -1 0 1", "50", "-du", "40", "--square-denominators"],
                    ["-2 0 1 0 1", "300", "-dl", "3", "-du", "90", "--square-denominators", "-y"]):
        code, expected, _, _ = oracle.run(["ratpoints_gpu", *command])
        assert rpg.cli(command).stdout == expected


def test_record_curve_published_points(rpg, golden):
    # tests/verify_record_curve.py: all 301 published x with height <= 10^6, nothing else
    rec = golden["record_curve"]
    result = rpg.cli([rec["coefficients"], rec["height"], "-q", "-y", "-i"])
    assert result.returncode == 0
    found = set()
    for line in result.stdout.decode().splitlines():
        a, b = line.strip("()").split(" : ")
        found.add(Fraction(int(a), int(b)))
    assert found == {Fraction(x) for x in rec["x"]}
    assert len(found) == 301


@pytest.mark.parametrize("index", [0, 1], ids=["b1e7", "b1e6"])
def test_record_curve_full_box(rpg, golden, index):
    # the reference's own full-box runs: stdout SHA-256 and exact points at height 10^7
    case = golden["record_full"][index]
    result = rpg.cli([case["coefficients"], case["height"], "-du", case["last"], "-v"])
    assert result.returncode == 0, result.stderr
    assert hashlib.sha256(result.stdout).hexdigest() == case["sha256"]
    if "bytes" in case:
        assert len(result.stdout) == case["bytes"]
    assert rpg.parse_metrics(result.stderr)["exact_survivors"] == case["exact_survivors"]


def test_record_curve_reference_plan_survivors(rpg, golden):
    # 32-prime plan on the full 10^7 box: the reference's modular survivor count
    case = golden["record_full"][0]
    result = rpg.cli([case["coefficients"], case["height"], "-v", "--sieve-plan", "reference"])
    assert result.returncode == 0, result.stderr
    assert hashlib.sha256(result.stdout).hexdigest() == case["sha256"]
    metrics = rpg.parse_metrics(result.stderr)
    assert metrics["survivors"] == case["reference_survivors"]
    assert metrics["exact_survivors"] == case["exact_survivors"]


def test_c1_configuration(rpg, golden):
    c1 = golden["c1"]
    for plan in ("reference", "fast"):
        result = rpg.cli([c1["coefficients"], c1["height"], "-du", c1["last"], "--sieve-plan", plan])
        assert result.returncode == 0
        assert hashlib.sha256(result.stdout).hexdigest() == c1["sha256"]


def test_devices_selection(rpg):
    base = rpg.cli(["1 0 1", "15"]).stdout
    assert rpg.cli(["1 0 1", "15", "--devices", "all"]).stdout == base
    assert rpg.cli(["1 0 1", "15", "--devices", "0"]).stdout == base
    listing = rpg.cli(["--list-devices"])
    assert listing.returncode == 0 and listing.stdout.startswith(b"device=0 name=")
    bad = rpg.cli(["1 0 1", "5", "--devices", "4096"])
    assert bad.returncode == 1 and b"is not visible" in bad.stderr


def test_large_coefficient_search_matches_oracle(rpg, oracle):
    import random
    rng = random.Random(31)
    coeffs = [str(rng.randint(-(2**200), 2**200)) for _ in range(21)]
    coeffs[0] = str(rng.randint(1, 2**100) ** 2)  # (0 : y : 1) is a point
    text = " ".join(coeffs)
    if not oracle.is_squarefree(coeffs):
        pytest.skip("random curve not squarefree")
    command = [text, "300", "-du", "40", "-l", "-1.5", "-u", "0.75", "-l", "2", "-u", "1e2"]
    code, expected, _, _ = oracle.run(["ratpoints_gpu", *command])
    assert code == 0 and expected
    assert rpg.cli(command).stdout == expected
