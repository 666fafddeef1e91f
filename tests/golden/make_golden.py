"""Generate the committed golden fixtures in tests/golden/ from the reference.

Run in a checkout where the reference tree is available, naming it with
--reference PATH (required).  Sources of truth:

* oracle_cases: the reference's independent Python oracle
  (tests/test_multi_gpu.py:17-40) imported from the reference tree and
  evaluated on its own cases (tests/test_multi_gpu.py:77-84) and on the
  point-search cases of tests/compare_with_ratpoints.py:17-30.
* dense: the multi-flush known answer (tests/test_multi_gpu.py:122-130,
  tests/compare_with_ratpoints.py:78-89): survivors=20002, exact_survivors=1.
* square_kat: tests of experiments/elliptic-curves/test_rank31_multifiber.py:75-81
  (the line "1 14 4" in the square-denominator search).
* record_curve: the published x-coordinates of tests/data/record_curve_x.txt
  with height <= 10^6 (tests/verify_record_curve.py:17-59).
* record_full: the record curve at height 10^7 with default options, as the
  reference's own measurement runs record it: denominators to 10^7 (stdout
  SHA-256, size and exact points, and the modular survivor count of the
  32-prime plan; docs/RTX4090-OPTIMIZATION.md:226-234) and to 10^6 (stdout
  SHA-256 and exact points; docs/RTX4090-SCREEN.json, variant "baseline").
* c1: a seeded degree-6 curve with coefficients in [-50, 50] on the box
  a in [-2000, 2000], b in [1, 2000]; expected output from the oracle pipeline
  (reference-plan sieve restated in C, exact verification in Python), pinned
  against the reference's Python oracle on the sub-box b <= 40.

    python tests/golden/make_golden.py [--reference PATH]
"""

from __future__ import annotations

import argparse
import hashlib
import json
import random
import re
import sys
from fractions import Fraction
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT / "oracle"))

import ratpoints_oracle as oracle  # noqa: E402

RECORD_CURVE = "247747600 -985905640 567207969 2396040466 52485681 -470135160 82342800"
C1_SEED = 20260950  # first seed from 20260917 whose C1 box holds >= 3 points


def c1_curve(seed=C1_SEED):
    rng = random.Random(seed)
    while True:
        coeffs = [rng.randint(-50, 50) for _ in range(7)]
        if coeffs[-1] != 0 and oracle.is_squarefree(coeffs):
            return " ".join(map(str, coeffs))


def pipeline_output(coefficients_text, height, first, last):
    argv = ["ratpoints_gpu", coefficients_text, str(height), "-dl", str(first), "-du", str(last)]
    code, out, err, _ = oracle.run(argv)
    assert code == 0, err
    return out


def main():
    parser = argparse.ArgumentParser(description=__doc__)
    parser.add_argument("--reference", required=True, help="root of the reference tree")
    args = parser.parse_args()
    ref = Path(args.reference)
    sys.path.insert(0, str(ref / "tests"))
    import test_multi_gpu as ref_tests  # the reference's own oracle module

    cases = []
    for coefficients, height, first, last in [
            ("1 0 1", 35, 1, 17), ("1 1 0 1", 35, 3, 15), ("1 0 1 0 1", 35, 1, 20),
            ("-3 5 -7 11 2", 35, 4, 19), ("+1 0 +1", 5, 1, 1),
            ("1 " + "0 " * 99 + "1", 7, 1, 3)]:
        expected = ref_tests.oracle(coefficients, height, first, last).decode()
        cases.append({"source": "tests/test_multi_gpu.py:77-84", "coefficients": coefficients,
                      "height": height, "first": first, "last": last, "stdout": expected})
    for coefficients, height, last in [
            ("1 0 1 0 1", 500, 40), ("-3 5 -7 11 2", 500, 40), ("1 1 0 1", 500, 40),
            ("+1 0 +1", 100, 20), ("1 " + "0 " * 99 + "1", 30, 10), (RECORD_CURVE, 1000, 200)]:
        expected = ref_tests.oracle(coefficients, height, 1, last).decode()
        cases.append({"source": "tests/compare_with_ratpoints.py:17-30", "coefficients": coefficients,
                      "height": height, "first": 1, "last": last, "stdout": expected})

    primes = [p for p in range(2, 512) if all(p % q for q in range(2, int(p ** 0.5) + 1))]
    p32 = 1
    for p in primes[-32:]:
        p32 *= p
    dense = {"coefficients": f"1 {p32}", "height": 5000, "first": 1, "last": 2,
             "survivors": 20002, "exact_survivors": 1,
             "stdout": ref_tests.oracle(f"1 {p32}", 5000, 1, 2).decode()}

    square_kat = {"args": ["1 -1 0 1", "10", "-dl", "1", "-du", "3", "--square-denominators",
                           "-i", "-f", "%x %y %z\\n"],
                  "contains": "1 14 4"}

    published = [Fraction(line) for line in
                 (ref / "tests" / "data" / "record_curve_x.txt").read_text().split()]
    within = sorted({x for x in published
                     if abs(x.numerator) <= 10 ** 6 and x.denominator <= 10 ** 6})
    record = {"coefficients": RECORD_CURVE, "height": 10 ** 6,
              "x": [f"{x.numerator}/{x.denominator}" for x in within]}

    text = (ref / "docs" / "RTX4090-OPTIMIZATION.md").read_text()
    shas = set(re.findall(r"SHA-256\s*`([0-9a-f]{64})`", text))
    assert len(shas) == 1, shas
    size = int(re.search(r"The output was ([0-9,]+)\s+bytes", text).group(1).replace(",", ""))
    row32 = re.search(r"^\| 32 \|.*\| ([0-9,]+) \|$", text, re.M).group(1)
    exact = set(int(n) for n in re.findall(r"([0-9]+) exact points", text))
    assert len(exact) == 1, exact
    screen = json.loads((ref / "docs" / "RTX4090-SCREEN.json").read_text())
    base = next(v for v in screen["variants"] if v["name"] == "baseline")
    record_full = [
        {"source": "docs/RTX4090-OPTIMIZATION.md:226-234", "coefficients": RECORD_CURVE,
         "height": 10 ** 7, "last": 10 ** 7, "sha256": shas.pop(), "bytes": size,
         "exact_survivors": exact.pop(), "reference_survivors": int(row32.replace(",", ""))},
        {"source": "docs/RTX4090-SCREEN.json", "coefficients": RECORD_CURVE,
         "height": base["height"], "last": base["denominator_max"], "sha256": base["output_sha256"],
         "exact_survivors": base["exact_survivors"]},
    ]

    c1 = c1_curve()
    c1_stdout = pipeline_output(c1, 2000, 1, 2000).decode()
    pin = ref_tests.oracle(c1, 2000, 1, 40).decode()
    sub = pipeline_output(c1, 2000, 1, 40).decode()
    assert pin == sub, "oracle pipeline disagrees with the reference oracle on the C1 sub-box"
    c1_fixture = {"coefficients": c1, "seed": C1_SEED, "height": 2000, "first": 1, "last": 2000,
                  "stdout": c1_stdout,
                  "sha256": hashlib.sha256(c1_stdout.encode()).hexdigest(),
                  "pinned_sub_box_last": 40}

    out = {"oracle_cases": cases, "dense": dense, "square_kat": square_kat,
           "record_curve": record, "record_full": record_full, "c1": c1_fixture}
    (HERE / "golden.json").write_text(json.dumps(out, indent=1) + "\n")
    print(f"wrote {HERE / 'golden.json'}: {len(cases)} oracle cases, "
          f"{len(within)} record-curve points, C1 curve {c1!r} "
          f"({c1_stdout.count(chr(10))} lines)")


if __name__ == "__main__":
    main()
