"""The tuning cache as a sieve reads it (host only): with RPG_TUNE_CACHE
naming a JSON file that holds a shape for a kind of curve, a fast-plan sieve
of a curve of that kind uses the stored shape; without the variable, with a
key of another kind of curve, or with a file that is not valid JSON, the
cost model decides.  The batch engine's work items per kernel are read the
same way, by kind of batch."""

import json
import math

import pytest

C2_LIKE = ["3101467171", "-2447016419", "1740004371", "-339009245", "4227431941", "-1204453621",
           "3517081707"]


def key_of(rpg, coeffs, bound):
    plan = rpg.fast_plan(coeffs, bound)
    largest = max((f for fs in plan["factors"] for f in fs), default=0)
    words = (2 * bound + 1 + 63) // 64
    return (f"degree{len(coeffs) - 1}-q{plan['class_prime']}-words2^{int(math.floor(math.log2(words)))}"
            f"-{'large' if largest >= 128 else 'small'}primes")


def test_cost_model_without_cache(rpg, monkeypatch):
    monkeypatch.delenv("RPG_TUNE_CACHE", raising=False)
    rows, slots, cached = rpg.fast_shape(C2_LIKE, 5_000_000)
    plan = rpg.fast_plan(C2_LIKE, 5_000_000)
    assert not cached and rows == len(plan["moduli"]) and slots == plan["slots"]


def test_stored_shape_is_used(rpg, monkeypatch, tmp_path):
    auto_rows, auto_slots, _ = rpg.fast_shape(C2_LIKE, 5_000_000)
    want_rows = auto_rows - 1 if auto_rows > 3 else auto_rows + 1
    want_slots = 2 if auto_slots == 3 else 3
    path = tmp_path / "shapes.json"
    path.write_text(json.dumps({"fast_plan_shapes": {
        key_of(rpg, C2_LIKE, 5_000_000): {"rows": want_rows, "slots": want_slots,
                                           "sample_denominators": 131072, "measured_ms": {}},
        "degree99-q1-words2^1-smallprimes": {"rows": 1, "slots": 2}}}))
    monkeypatch.setenv("RPG_TUNE_CACHE", str(path))
    rows, slots, cached = rpg.fast_shape(C2_LIKE, 5_000_000)
    assert cached and rows == want_rows and slots == want_slots
    # another kind of curve (degree 4) keeps the cost model's shape
    other = ["1", "0", "-7", "0", "13"]
    rows, slots, cached = rpg.fast_shape(other, 5_000_000)
    assert not cached


def test_unreadable_cache_is_ignored(rpg, monkeypatch, tmp_path):
    path = tmp_path / "broken.json"
    path.write_text('{"fast_plan_shapes": {"degree6": {"rows": ')
    monkeypatch.setenv("RPG_TUNE_CACHE", str(path))
    rows, slots, cached = rpg.fast_shape(C2_LIKE, 5_000_000)
    assert not cached
    monkeypatch.setenv("RPG_TUNE_CACHE", str(tmp_path / "missing.json"))
    assert not rpg.fast_shape(C2_LIKE, 5_000_000)[2]


def test_tuner_rejects_bad_arguments(rpg):
    import pytest
    with pytest.raises(rpg.RpgError):
        rpg.tune_fast_plan(C2_LIKE, 1000, 5, 4)
    with pytest.raises(rpg.RpgError):
        rpg.tune_fast_plan(C2_LIKE, 0, 1, 4)


def batch_key(curves):
    words = sorted((2 * c["bound"] + 1 + 63) // 64 for c in curves)
    degrees = sorted(len(c["coefficients"]) - 1 for c in curves)
    n = len(curves)
    return (f"curves2^{int(math.floor(math.log2(n)))}-words2^{int(math.floor(math.log2(words[n // 2])))}"
            f"-degree-{'low' if degrees[n // 2] <= 6 else 'high'}")


BATCH = [{"coefficients": ["1", "0", "0", "17"][::-1], "bound": 70000 + 1000 * i, "first": 1, "last": 5}
         for i in range(5)] + [{"coefficients": ["1", "2", "3", "4", "5", "6", "7", "8", "9"], "bound": 500,
                                "first": 1, "last": 9}]


def test_batch_items_default_and_stored(rpg, monkeypatch, tmp_path):
    # without a cache file: 8,192 work items per kernel; with one holding this
    # kind of batch (curve count, median row length, median degree), its value,
    # next to the fast-plan shapes of the same file
    monkeypatch.delenv("RPG_TUNE_CACHE", raising=False)
    assert rpg.batch_items(BATCH) == (8192, False)
    path = tmp_path / "tuning.json"
    path.write_text(json.dumps({
        "fast_plan_shapes": {key_of(rpg, C2_LIKE, 5_000_000): {"rows": 5, "slots": 2}},
        "batch_items": {batch_key(BATCH): {"items": 2048, "measured_ms": {"2048": 1.0, "8192": 1.5}},
                        batch_key(BATCH[:1]): {"items": 32768}}}))
    monkeypatch.setenv("RPG_TUNE_CACHE", str(path))
    assert rpg.batch_items(BATCH) == (2048, True)
    assert rpg.fast_shape(C2_LIKE, 5_000_000)[2]
    # another kind of batch (one curve) finds its own entry; a degree-10 batch none
    assert rpg.batch_items(BATCH[:1]) == (32768, True)
    high = [dict(c, coefficients=[str(v) for v in range(11)]) for c in BATCH]
    assert rpg.batch_items(high) == (8192, False)


def test_batch_items_unreadable_cache(rpg, monkeypatch, tmp_path):
    path = tmp_path / "broken.json"
    path.write_text('{"batch_items": {"' + batch_key(BATCH) + '": {"items": ')
    monkeypatch.setenv("RPG_TUNE_CACHE", str(path))
    assert rpg.batch_items(BATCH) == (8192, False)
    with pytest.raises(rpg.RpgError):
        rpg.tune_batch([])


def test_batch_stats_fields(rpg):
    stats = rpg.BatchStats().as_dict()
    assert {"items_per_kernel", "items_from_cache", "swept_words", "smem_bytes"} <= set(stats)
