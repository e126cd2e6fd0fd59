"""bench.py's JSON line without a GPU: the GB300 arm driven by a stand-in engine that returns
fixed timings, checked for every key the benchmark contract asks for; and the reference arm
(the oracle port on the host cores) on a short run."""
import importlib
import json
import os
import sys

import pytest

from conftest import ROOT

TIMING = {"total_ms": 1.5, "mark_ms": 1.0, "mr_ms": 0.09, "rung_ms": 0.39, "direct_ms": 0.006, "prep_ms": 0.015,
          "mark_short_ms": 0.98, "mark_long_ms": 0.007, "marks_kernel_launches": 1, "kernel_launches": 7,
          "mark_items": 0, "survivors": 370000, "primes": 1632, "short_pairs": 0, "mask_bytes": 2308 * 33408,
          "host_setup_ms": 0.11, "host_device_ms": 1.53, "host_collect_ms": 0.05, "host_total_ms": 1.77}


class StandInEngine:
    """The Engine methods bench.py calls, with fixed answers (no device)."""

    def __init__(self, **kw):
        self.closed = False

    def autotune(self, windows, repeats=6):
        return self.schedule()

    def schedule(self):
        return {"short_max": 64, "rung_blocks_per_sm": 6, "long_split": 1}

    def run_batch(self, windows, schedule=1, records=True):
        import numpy as np
        import es_sieve
        return [{"rung": 0} for _ in windows], (np.zeros(3, dtype=es_sieve.RECORD_DTYPE) if records else None)

    def submit_batch_c(self, warr, n):
        return 1

    def poll_c(self, ticket, carr, timeout_ms=-1):
        return 1632

    def make_windows(self, windows):
        return windows

    def make_counters(self, n):
        return None

    def run_batch_c(self, warr, n, carr, schedule=1):
        return 1632

    def run_window(self, lo, hi):
        return {}, []

    def timing(self):
        return dict(TIMING)

    def close(self):
        self.closed = True

    def set_schedule(self, **kw):
        pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def _bench(monkeypatch, argv):
    sys.path.insert(0, ROOT)
    import es_sieve
    monkeypatch.setattr(es_sieve, "Engine", StandInEngine)
    bench = importlib.import_module("bench")
    monkeypatch.setattr(sys, "argv", ["bench.py"] + argv)
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    return bench


def test_gpu_arm_line_has_every_contract_key(monkeypatch, capsys):
    bench = _bench(monkeypatch, ["--steps", "2", "--warmup", "3", "--serve", "0", "--no-cpu-baseline"])
    # ncu figures for the stand-in's schedule only: the issue fraction must use them
    monkeypatch.setattr(bench, "MARK_SHORT_NCU", {(64, 1): {"inst": 8e8, "dram": 82e6}})
    monkeypatch.setattr(bench, "RUNG_NCU", {6: {"inst": 1.2e8, "dram": 1e6}})
    bench.main()
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "e2e", "gpu_launches", "clocks", "roofline", "cpu_baseline"):
        assert k in line, k
    assert line["n_gpus"] == 1 and line["steps"] == 2 and line["warmup"] == 3 and line["higher_is_better"]
    assert line["config"]["workload"] == "batch4096" and "l2" in line["config"]
    assert abs(line["ms_per_step"] - TIMING["total_ms"]) < 1e-9
    assert abs(line["value"] - line["config"]["integers_per_step"] / (TIMING["total_ms"] / 1000)) < 1
    for k in ("value", "unit", "h2d_bytes_per_step", "d2h_bytes_per_step"):
        assert k in line["e2e"], k
    assert "mode" in line["e2e"] and line["e2e_sync"]["value"] > 0
    assert line["gpu_launches"] == 2 * 2 * TIMING["kernel_launches"]       # the synchronous and pipelined steps
    roof = line["roofline"]
    for k in ("bound", "achieved", "peak", "unit", "frac", "traffic"):
        assert k in roof, k
    assert roof["kernel"] == "k_mark_short" and roof["bound"] == "issue" and roof["unit"] == "warp inst/s"
    assert abs(roof["frac"] - roof["achieved"] / roof["peak"]) < 1e-12 and 0 < roof["frac"] < 2
    assert roof["traffic"] == 82e6 and roof["schedule"] == StandInEngine().schedule()
    assert 0 < roof["hbm"]["frac"] < 1 and roof["hbm"]["unit"] == "GB/s"
    assert 0 < roof["stage_d"]["issue"]["frac"] < 2
    assert set(line["clocks"]) >= {"sm_mhz", "sm_max_mhz", "reasons"}
    assert line["plain"]["records_identical"] and "c3" in line
    g = line["gb300_table"]
    assert g["filters"] > 3745 and g["batch4096"]["value"] > 0 and g["batch19"]["e2e"]["value"] > 0
    b19 = line["batch19"]
    assert b19["windows"] == 4096 and b19["value"] > 0 and b19["e2e"]["value"] > 0 and b19["plain"]["value"] > 0
    assert line["e2e_host_ms_per_step"]["total_ms"] == pytest.approx(TIMING["host_total_ms"])


def test_roofline_without_a_capture_for_the_schedule(monkeypatch, capsys):
    bench = _bench(monkeypatch, ["--steps", "1", "--warmup", "3", "--serve", "0", "--no-cpu-baseline", "--no-plain",
                                 "--no-batch19"])
    monkeypatch.setattr(bench, "MARK_SHORT_NCU", {(128, 1): {"inst": 8e8, "dram": 82e6}})
    bench.main()
    roof = json.loads(capsys.readouterr().out.strip().splitlines()[-1])["roofline"]
    assert roof["achieved"] is None and roof["frac"] is None and "note" in roof


def test_reference_arm_line(monkeypatch, capsys):
    bench = _bench(monkeypatch, ["--impl", "reference", "--steps", "1", "--warmup", "1", "--cpu-windows", "3"])
    bench.main()
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] == os.cpu_count()
    assert line["e2e"] == {"value": line["value"], "unit": "integers/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
