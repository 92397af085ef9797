"""CPU tests of bench.py's host-side helpers (no GPU)."""
import json

import bench


def test_summary_collects_every_form_and_tolerates_missing_ones():
    line = {"ms_per_step": 0.042, "parity_with_oracle": True,
            "e2e": {"ms_per_step": 0.045, "one_in_flight_ms_per_step": 0.063},
            "roofline": {"frac": 0.036}, "plain_small": {"ms_per_step": 0.012, "parity_with_oracle": True,
                                                        "roofline": {"frac": 0.12}},
            "batched": None, "stress": {"views_per_s": 2.6e5, "parity": True},
            "served": {"max_sustained_views_per_s": 8e4,
                       "runs": [{"rate": 2000.0, "latency_p50_ms": 0.2, "latency_p99_ms": 0.4}]}}
    s = bench.run_summary(line)
    assert s["plain_large_ms_per_step"] == 0.042 and s["plain_small_frac"] == 0.12
    assert s["batch_views_per_s"] is None and s["stress_parity"] is True
    assert s["served_p50_p99_ms"] == {"2000": [0.2, 0.4]}
    json.dumps(s)  # serialisable


def test_fp32_peak_uses_the_device_sm_count():
    assert abs(bench.fp32_peak_tops(152, 2070.0) - 40.27392) < 1e-9
    assert abs(bench.fp32_peak_tops(148, 1965.0) - 148 * 128 * 1965e6 / 1e12) < 1e-9
