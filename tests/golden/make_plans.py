"""Generate tests/golden/plans.json: the fast-plan autotuner's decisions
(rpg_fast_plan) for seeded curves and heights.

This is a regression fixture of this project's own planner, not a reference
pin: the fast plan has no counterpart in the reference (its 32-prime plan is
fixed).  Planner changes meant to be pure speed-ups must leave it unchanged;
changes to the plan itself regenerate it.

    python tests/golden/make_plans.py
"""

from __future__ import annotations

import json
import random
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "ratpoints-gpu_gb300"))


def cases():
    rng = random.Random(20261203)
    out = []
    for _ in range(60):
        degree = rng.choice([1, 2, 3, 4, 5, 6, 8, 10, 16])
        bits = rng.choice([4, 16, 32, 64, 200])
        coeffs = [rng.randint(-(2**bits), 2**bits) for _ in range(degree + 1)]
        if coeffs[-1] == 0:
            coeffs[-1] = 1
        height = rng.choice([10, 1000, 10**5, 5 * 10**6, 10**8, 10**10])
        out.append({"coefficients": " ".join(map(str, coeffs)), "height": height})
    return out


def main():
    import ratpoints_gb300 as rpg

    rows = []
    for case in cases():
        plan = rpg.fast_plan(case["coefficients"], case["height"])
        rows.append({**case, "plan": plan})
    path = Path(__file__).with_name("plans.json")
    path.write_text(json.dumps(rows, indent=1) + "\n")
    print(f"{len(rows)} plans -> {path}")


if __name__ == "__main__":
    main()
