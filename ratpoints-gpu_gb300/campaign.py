"""Many-curve searches in one batched call, for research campaigns.

The reference's campaign scripts run the ratpoints_gpu binary once per curve
(experiments/elliptic-curves/rank31_family_hunt.py:131-155 builds
``ratpoints_gpu '<c0 .. cn>' H -dl DL -du DU --batch-size 65536 -i -v [-z]``
and reads ``exact_survivors=`` and ``survivors=`` from the -v line and the
points from stdout).  ``search_many`` takes the same per-curve arguments, runs
all curves in one ``rpg_batch_search`` call (tables resident, two persistent
kernels, one CUDA graph) and returns per curve what those scripts read:

* ``exact_survivors``: verified (a, b) pairs, as the -v line counts them;
* ``points``: [(a, y, b)], y >= 0, in the command line's order;
* ``stdout``: the lines the command line prints with -i (points at infinity
  left out unless asked for), each point as ``(a : y : b)`` then
  ``(a : -y : b)`` when y != 0;
* ``modular_survivors``: the batch plan's modular survivors.  Like the
  command line's fast plan (and unlike ``--sieve-plan reference``), this
  count depends on the plan, so it is reported but not comparable across
  plans; the points are the same whatever the plan.
"""

from __future__ import annotations

import time

import ratpoints_gb300 as rpg


def format_points(points, include_infinity=False):
    """Default command-line output lines of a point list (src/output_formatter.cpp)."""
    lines = []
    for a, y, b in points:
        if b == 0 and not include_infinity:
            continue
        lines.append(f"({a} : {y} : {b})\n")
        if y != 0:
            lines.append(f"({a} : {-y} : {b})\n")
    return "".join(lines)


def search_many(requests, device=-1, include_infinity=False):
    """requests: iterable of dicts with ``coefficients`` (list or text),
    ``height`` and optional ``dl`` (default 1), ``du`` (default height),
    ``square`` (square denominators).  Returns (results, seconds): one dict
    per request, in order, and the wall time of the batched call."""
    curves = []
    for r in requests:
        coeffs = rpg.coefficients_of(r["coefficients"])
        height = int(r["height"])
        curves.append({"coefficients": coeffs, "bound": height, "first": int(r.get("dl", 1)),
                       "last": int(r.get("du", height)), "square": bool(r.get("square", False)),
                       "include_infinity": include_infinity})
    started = time.perf_counter()
    points, status, survivors, _ = rpg.batch_search(curves, device=device)
    seconds = time.perf_counter() - started
    results = []
    for c, pts, st, surv in zip(curves, points, status, survivors):
        finite = [p for p in pts if p[2] != 0]
        results.append({"status": st, "coefficients": c["coefficients"], "height": c["bound"],
                        "exact_survivors": len(finite), "modular_survivors": surv,
                        "points": pts, "stdout": format_points(pts, include_infinity)})
    return results, seconds
