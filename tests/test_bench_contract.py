"""Host-side pieces of bench.py that need no GPU: a secondary workload that
fails is recorded with its error instead of ending the run, so the headline
JSON line still prints."""
from __future__ import annotations

import argparse
import os
import sys

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


def test_failing_workloads_are_recorded_not_raised(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench

    def boom(*a, **k):
        raise RuntimeError("no device")

    for name in ("run_batched", "run_served", "run_wide", "run_exact_forms"):
        monkeypatch.setattr(bench, name, boom)
    out = bench.other_workloads(argparse.Namespace(steps=5, warmup=3))
    assert set(out) == {"batched", "served", "wide", "exact_fallback"}
    assert all(v == {"error": "RuntimeError: no device"} for v in out.values())


def test_default_arguments_fit_the_timing_rules():
    sys.path.insert(0, ROOT)
    import bench

    saved = sys.argv
    sys.argv = ["bench.py"]
    try:
        args = bench.parse_args()
    finally:
        sys.argv = saved
    assert args.warmup >= 3 and args.steps >= 1 and args.gpus == 1 and args.workload == "chunk"


def test_workload_records_are_summarised(monkeypatch):
    """The compact records built from each workload's full line (stub lines
    with the fields the full runs emit)."""
    sys.path.insert(0, ROOT)
    import bench

    lat = {"latency_ms": {"p50": 0.1, "p99": 0.2, "p99.9": 0.3}, "beam_samples_per_s": 1e9, "mismatches": 0}
    batched = {"config": {"workload": "b"}, "value": 1.0, "unit": "u", "ms_per_step": 0.35,
               "roofline": {"frac": 0.46, "bound": "hbm"}, "speedup_vs_per_problem": 4.3,
               "autotune": {"launches": [{"problems": 26, "max_nb_pass": 96, "ctas_per_sm": 1}]},
               "parity": "ok"}
    served = {"config": {"workload": "s for 30 s"}, "served": lat, "plain_loop": lat, "served_saturation": lat,
              "plain_saturation": lat, "p99_ratio_plain_over_served": 1.5, "saturation_speedup": 2.0,
              "clocks": None}
    wide = {"config": {"workload": "w"}, "value": 2.0, "unit": "u", "ms_per_step": 0.86,
            "roofline": {"frac": 0.6, "bound": "tensor", "kernel_ms": 0.75}, "served": {"weight_updates": 48},
            "mismatches": 0, "clocks": None}
    monkeypatch.setattr(bench, "run_batched", lambda a, emit=True: batched)
    monkeypatch.setattr(bench, "run_served", lambda a, emit=True: served)
    monkeypatch.setattr(bench, "run_wide", lambda a, emit=True: wide)
    monkeypatch.setattr(bench, "run_exact_forms", lambda: {"gauss_speedup": 2.0})
    out = bench.other_workloads(argparse.Namespace(steps=5, warmup=3))
    assert not any("error" in v for v in out.values()), out
    assert out["batched"]["launches"] == [(26, 96, 1)]
    assert out["served"]["workload"] == "s for 10 s" and out["served"]["mismatches"] == 0
    assert out["wide"]["kernel_ms"] == 0.75 and out["exact_fallback"]["gauss_speedup"] == 2.0
