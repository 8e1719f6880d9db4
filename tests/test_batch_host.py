"""Host logic of batched compression (seemps2_gb300.batch) without a GPU: the report's rate,
percentiles (nearest rank on the sorted latencies) and summary fields."""

import pytest

batch = pytest.importorskip("seemps2_gb300.batch")


def test_report_rate_and_percentiles():
    lat = [0.5, 0.1, 0.4, 0.2, 0.3]
    rep = batch.BatchReport(streams=4, wall_s=2.0, latencies_s=lat)
    assert rep.instances_per_s == pytest.approx(2.5)
    assert rep.percentile(0) == 0.1
    assert rep.percentile(50) == 0.3
    assert rep.percentile(100) == 0.5
    assert rep.percentile(99) == 0.5  # round(0.99 * 4) = 4
    s = rep.summary()
    assert s["streams"] == 4 and s["instances"] == 5
    assert s["p50_s"] == 0.3 and s["p99_s"] == 0.5
    assert s["mean_s"] == pytest.approx(0.3)


def test_empty_report():
    rep = batch.BatchReport(streams=1, wall_s=0.0)
    assert rep.instances_per_s == 0.0
    assert rep.percentile(50) == 0.0
    assert rep.summary()["mean_s"] == 0.0
