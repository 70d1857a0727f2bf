"""bench.py's roofline arithmetic on CPU: the seeding + lookup stage against the HBM copy
bandwidth and the random-gather ceiling, the whole batch's algorithmic bytes, and the
per-configuration DRAM traffic of the committed ncu summaries."""
import os
import sys

import pytest

sys.path.insert(0, os.path.join(os.path.dirname(__file__), ".."))

import bench  # noqa: E402


def test_lookup_roofline_fused_and_two_kernel_forms():
    peak, _ = bench.peaks()
    # fused (seeding + lookup one kernel): the packed reads count with the probes
    r = bench.lookup_roofline(alg_lookup=5_000_000_000, sectors=250_000_000, packed=76_000_000, nams=24_000_000,
                              stage_ms={"seed_lookup": 5.0, "nams": 3.0}, fused=True, ms=13.0, gather_gbs=3000.0)
    assert r["kernel"] == "seed_lookup" and r["alg_bytes_per_launch"] == 5_076_000_000
    assert r["achieved"] == pytest.approx(5_076_000_000 / 5e-3 / 1e9, abs=0.1)
    assert r["frac"] == pytest.approx(r["achieved"] / peak, abs=1e-4)
    assert r["gather"]["achieved"] == pytest.approx(250_000_000 * 32 / 5e-3 / 1e9, abs=0.1)
    assert r["gather"]["frac"] == pytest.approx(1600.0 / 3000.0, abs=1e-4)
    whole = 76_000_000 + 5_000_000_000 + 44 * 24_000_000
    assert r["whole_batch"]["alg_bytes"] == whole
    assert r["whole_batch"]["frac"] == pytest.approx(whole / 13e-3 / 1e9 / peak, abs=1e-4)
    # two kernels (indexes over 2 GiB): the lookup kernel carries the probes alone
    r = bench.lookup_roofline(alg_lookup=26_000_000_000, sectors=1_400_000_000, packed=380_000_000,
                              nams=96_000_000, stage_ms={"seed": 18.0, "lookup": 36.0}, fused=False, ms=84.0,
                              gather_gbs=1200.0)
    assert r["kernel"] == "lookup" and r["alg_bytes_per_launch"] == 26_000_000_000
    assert r["gather"]["frac"] == pytest.approx(1_400_000_000 * 32 / 36e-3 / 1e9 / 1200.0, abs=1e-4)
    # a stage that did not run gives no rate
    r = bench.lookup_roofline(1, 1, 1, 1, {}, True, 1.0, 1.0)
    assert r["achieved"] is None and r["frac"] is None and r["gather"]["frac"] is None


def test_ncu_traffic_is_per_configuration():
    c2 = bench.ncu_traffic("C2")
    c4 = bench.ncu_traffic("C4")
    assert c2["seed_lookup"] > 0 and "lookup" not in c2
    assert c4["lookup"] > c4["seed"] > 0
    assert bench.ncu_traffic("C1") == {} and bench.ncu_traffic("C3") == {}
