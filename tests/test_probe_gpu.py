"""rpg_smem_read_probe, the denominator of the sieve's shared-memory
roofline: it runs, its two measures agree with each other, and they lie in
the range a GB300 SM can deliver (nominal 128 B/clk/SM of shared loads)."""

import pytest

pytestmark = pytest.mark.gpu


def test_probe_measures_a_plausible_rate(rpg):
    r = rpg.smem_read_probe(iterations=2048)
    assert r["ms"] > 0
    assert 32.0 <= r["bytes_per_clock_per_sm"] <= 160.0, r
    # GB/s over 152 SMs at a clock between 1.0 and 2.2 GHz
    implied_ghz = r["gbs"] / (152 * r["bytes_per_clock_per_sm"])
    assert 0.9 <= implied_ghz <= 2.3, r


def test_probe_rejects_bad_arguments(rpg):
    with pytest.raises(rpg.RpgError):
        rpg.smem_read_probe(iterations=0)
