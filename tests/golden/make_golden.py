"""Generate the committed golden fixtures in tests/golden/ from the reference.

Run in a checkout where the reference tree is available (default
/root/reference, or --reference PATH).  Sources of truth:

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
    parser.add_argument("--reference", default="/root/reference")
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
           "record_curve": record, "c1": c1_fixture}
    (HERE / "golden.json").write_text(json.dumps(out, indent=1) + "\n")
    print(f"wrote {HERE / 'golden.json'}: {len(cases)} oracle cases, "
          f"{len(within)} record-curve points, C1 curve {c1!r} "
          f"({c1_stdout.count(chr(10))} lines)")


if __name__ == "__main__":
    main()
