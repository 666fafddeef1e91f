"""The measured tuner of the fast plan's shape on the GPU: it times the cost
model's shape and its neighbours, reports the fastest, stores it in the
RPG_TUNE_CACHE file, and a later search of the same curve uses the stored
shape with the same points as the cost model's plan."""

import json

import pytest

pytestmark = pytest.mark.gpu


def test_tuner_measures_stores_and_is_used(rpg, monkeypatch, tmp_path):
    import bench
    coeffs = bench.c2_curve()
    bound, first, last = 400_000, 1, 30_000
    path = tmp_path / "shapes.json"
    monkeypatch.setenv("RPG_TUNE_CACHE", str(path))
    report = rpg.tune_fast_plan(coeffs, bound, first, last, sample=20_000)
    assert report["stored"] and report["sample"] == 20_000
    cands = report["candidates"]
    assert len(cands) >= 3
    best = min(cands, key=lambda c: c["ms"])
    assert (report["rows"], report["slots"]) == (best["rows"], best["slots"])
    assert all(c["ms"] > 0 for c in cands)
    stored = json.loads(path.read_text())["fast_plan_shapes"][report["key"]]
    assert (stored["rows"], stored["slots"]) == (report["rows"], report["slots"])
    assert len(stored["measured_ms"]) == len(cands)
    rows, slots, cached = rpg.fast_shape(coeffs, bound)
    assert cached and (rows, slots) == (report["rows"], report["slots"])
    with rpg.Session(coeffs, bound, plan="fast") as session:
        _, primes = session.plan()
    assert len(primes) >= rows  # the stored row count (rows of prime products)
    tuned, _ = rpg.point_search(coeffs, bound, first, last)
    monkeypatch.delenv("RPG_TUNE_CACHE")
    plain, _ = rpg.point_search(coeffs, bound, first, last)
    assert tuned == plain


def test_tuner_on_a_dense_curve_keeps_points(rpg, golden, monkeypatch, tmp_path):
    rec = golden["record_curve"]["coefficients"].split()
    monkeypatch.setenv("RPG_TUNE_CACHE", str(tmp_path / "dense.json"))
    report = rpg.tune_fast_plan(rec, 100_000, 1, 3000, sample=3000)
    assert report["key"].endswith("largeprimes")
    tuned, _ = rpg.point_search(rec, 100_000, 1, 3000)
    monkeypatch.delenv("RPG_TUNE_CACHE")
    plain, _ = rpg.point_search(rec, 100_000, 1, 3000)
    assert tuned == plain and plain


def test_batch_tuner_measures_stores_and_is_used(rpg, monkeypatch, tmp_path):
    # the batch engine's work items per kernel: three targets timed, the
    # fastest stored under the kind of batch and used by the next batch of
    # that kind, with the same points as the default
    import workloads
    curves = workloads.mixed_batch(96)
    path = tmp_path / "tuning.json"
    monkeypatch.setenv("RPG_TUNE_CACHE", str(path))
    report = rpg.tune_batch(curves)
    cands = report["candidates"]
    assert [c["items"] for c in cands] == [2048, 8192, 32768] and all(c["ms"] > 0 for c in cands)
    assert report["items"] == min(cands, key=lambda c: c["ms"])["items"] and report["stored"]
    stored = json.loads(path.read_text())["batch_items"][report["key"]]
    assert stored["items"] == report["items"] and len(stored["measured_ms"]) == 3
    assert rpg.batch_items(curves) == (report["items"], True)
    tuned, status, _, stats = rpg.batch_search(curves)
    assert stats["items_per_kernel"] == report["items"] and stats["items_from_cache"] == 1
    monkeypatch.delenv("RPG_TUNE_CACHE")
    plain, status2, _, stats2 = rpg.batch_search(curves)
    assert stats2["items_per_kernel"] == 8192 and not stats2["items_from_cache"]
    assert tuned == plain and status == status2
