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
