"""The GB300-tuned filter table on the device, pinned to the reference's scanner run on it.

tests/golden/gen/*_gb300.* were written by tests/golden/make_fixtures.py with the reference's
own sweep_lane (ref_sweep --filters erdos-strauss_gb300/tables/f_M2042040_mmax2000_gb300.txt):
the mid-height and top-of-range 2^34 shards byte for byte, and both 4096-window batches window
by window (SUMMARY and the sha256 of the records) under both launch schedules."""
import os

import pytest

import es_sieve
import workloads
from conftest import PKG, golden, read
from test_gpu_pinned import window_digests

pytestmark = pytest.mark.gpu

TABLE = os.path.join(PKG, "tables", "f_M2042040_mmax2000_gb300.txt")
_eng = []


def engine():
    if not _eng:
        _eng.append(es_sieve.Engine(wheel=2042040, filters=TABLE))
    return _eng[0]


@pytest.mark.parametrize("name", ["c2", "c3"])
def test_2p34_shards_byte_identical(name):
    c = workloads.c2() if name == "c2" else workloads.c3()
    assert engine().stream(c["lo"], c["hi"]) == read("gen", name + "_gb300.out")


@pytest.mark.parametrize("name", ["batch4096", "batch19_4096"])
def test_every_window_of_the_batch_matches_the_reference(name):
    wins = workloads.read_windows(golden("gen", name + ".windows"))
    rows = []
    for ln in read("gen", name + "_gb300.digests").splitlines(keepends=True):
        h, n, summ = ln.split(" ", 2)
        rows.append((h, int(n), summ))
    assert len(rows) == len(wins) == 4096
    eng = engine()
    for sched in (es_sieve.ES_SCHED_PERSISTENT, es_sieve.ES_SCHED_PLAIN):
        per, recs = eng.run_batch(wins, schedule=sched)
        got = window_digests(eng, wins, per, recs)
        bad = [i for i in range(len(wins)) if got[i] != rows[i]]
        assert not bad, (sched, bad[:5])


def test_tuner_measures_prefix_tables_on_the_gpu(tmp_path):
    """filter_tune.py --measure: two prefix tables through the engine, one timed call each;
    the calibration file it writes holds the per-kernel times and the counts the fit reads, and
    the longer prefix leaves fewer survivors."""
    import json
    import subprocess
    import sys
    out = tmp_path / "cal.json"
    r = subprocess.run([sys.executable, os.path.join(PKG, "filter_tune.py"), "--prefixes", "96,160", "--out",
                        str(tmp_path), "--measure", str(out), "--measure-steps", "1"],
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    rows = json.load(open(out))["rows"]
    assert [row["k"] for row in rows] == [96, 160]
    for row in rows:
        assert row["mark_short_ms"] > 0 and row["mr_ms"] > 0 and row["rung_ms"] > 0
    assert rows[1]["survivors"] < rows[0]["survivors"] and rows[1]["primes"] < rows[0]["primes"]

