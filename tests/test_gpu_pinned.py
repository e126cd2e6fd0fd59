"""Whole workloads pinned to the reference, on the GPU.

* Both 4096-window batches the bench times (heights log-uniform from the floor, and at the top
  of the range), every window: its SUMMARY line and the sha256 of its record lines must equal
  what the reference's own sweep_lane produced for it (tests/golden/gen/*.digests, written by
  tests/golden/make_fixtures.py from ref_sweep --windows), under both launch schedules.
* The reference's w64 window (data/rederive/windows/): the top 10^15 integers below the stage-E
  ceiling, 8,284,620 certificates. Through the drop-in binary in the production driver's order:
  SUMMARY byte-equal, the first and last 2,000 certificates equal, and both published stream
  digests (full stdout, certificates only) equal; then every record re-checked on the device.
"""
import collections
import hashlib

import numpy as np
import pytest

import es_sieve
import workloads
from conftest import golden, read

pytestmark = pytest.mark.gpu

GPU = golden("filters", "f_M2042040_mmax2000_gpu.txt")
W64 = (18445744065119614976, 18446744065119614976)

_eng = []


def engine():
    if not _eng:
        _eng.append(es_sieve.Engine(wheel=2042040, filters=GPU))
    return _eng[0]


def pinned(name):
    """(windows, [(sha256, n_records, SUMMARY line)]) of a committed batch fixture."""
    wins = workloads.read_windows(golden("gen", name + ".windows"))
    rows = []
    for ln in read("gen", name + ".digests").splitlines(keepends=True):
        h, n, summ = ln.split(" ", 2)
        rows.append((h, int(n), summ))
    assert len(wins) == len(rows) == 4096
    return wins, rows


def window_digests(eng, wins, per, recs):
    order = np.argsort(recs["window"], kind="stable")
    recs = recs[order]
    bounds = np.searchsorted(recs["window"], np.arange(len(wins) + 1))
    out = []
    for i, (lo, hi) in enumerate(wins):
        text = "".join(es_sieve.format_record(r) for r in recs[bounds[i]:bounds[i + 1]])
        out.append((hashlib.sha256(text.encode()).hexdigest(), int(bounds[i + 1] - bounds[i]),
                    eng.summary(lo, hi, per[i])))
    return out


@pytest.mark.parametrize("name", ["batch4096", "batch19_4096"])
def test_every_window_of_the_batch_matches_the_reference(name):
    wins, rows = pinned(name)
    eng = engine()
    for sched in (es_sieve.ES_SCHED_PERSISTENT, es_sieve.ES_SCHED_PLAIN):
        per, recs = eng.run_batch(wins, schedule=sched)
        got = window_digests(eng, wins, per, recs)
        bad = [i for i in range(len(wins)) if got[i] != rows[i]]
        assert not bad, (sched, bad[:5], [got[i] for i in bad[:2]], [rows[i] for i in bad[:2]])
    assert sum(r[1] for r in rows) > 1000


def test_pipelined_batches_match_the_reference():
    """es_submit_batch with three batches in flight on the two serving streams (each batch's
    marking chained after the previous one's, its stage D beside the next marking), the two
    pinned batches alternating: every window of every batch still gives the reference's
    SUMMARY and record digest."""
    eng = engine()
    names = ["batch4096", "batch19_4096"] * 3
    data = {n: pinned(n) for n in set(names)}
    tickets, done = [], []
    for name in names:
        tickets.append((name, eng.submit_batch(data[name][0])))
        if len(tickets) >= 3:
            n0, t0 = tickets.pop(0)
            done.append((n0, eng.poll(t0, 4096, timeout_ms=120000)))
    for n0, t0 in tickets:
        done.append((n0, eng.poll(t0, 4096, timeout_ms=120000)))
    assert [n for n, _ in done] == names
    for name, (per, recs) in done:
        wins, rows = data[name]
        got = window_digests(eng, wins, per, recs)
        bad = [i for i in range(len(wins)) if got[i] != rows[i]]
        assert not bad, (name, bad[:5])


def test_batch_fixture_windows_are_the_seeded_workloads():
    """The committed windows are what workloads.py draws on this machine (the bench reads the
    committed file, so a libm that rounds differently cannot change what is timed)."""
    assert workloads.read_windows(golden("gen", "batch4096.windows")) == workloads.batch_windows(4096)
    assert workloads.read_windows(golden("gen", "batch19_4096.windows")) == workloads.batch19_windows(4096)


def test_w64_top_of_range_window_through_the_cli():
    import subprocess
    digests = dict(ln.split()[::-1] for ln in read("windows", "w64.sha256").splitlines() if ln.strip())
    head_want = read("windows", "w64_head.txt").splitlines(keepends=True)
    tail_want = read("windows", "w64_tail.txt").splitlines(keepends=True)
    summary_want = read("windows", "w64_summary.txt")
    p = subprocess.Popen([es_sieve.CLI_PATH, str(W64[0]), str(W64[1]), "--filters", GPU, "--order", "round"],
                         stdout=subprocess.PIPE, stderr=subprocess.PIPE)
    full, certs = hashlib.sha256(), hashlib.sha256()
    head, tail, summary, n = [], collections.deque(maxlen=2000), None, 0
    for ln in p.stdout:
        full.update(ln)
        if ln.startswith(b"SUMMARY "):
            summary = ln.decode()
            continue
        certs.update(ln)
        n += 1
        s = ln.decode()
        if len(head) < 2000:
            head.append(s)
        tail.append(s)
    err = p.stderr.read().decode()
    assert p.wait() == 0, err
    assert summary == summary_want
    assert n == 8284620
    assert head == head_want
    assert list(tail) == tail_want
    assert certs.hexdigest() == digests["w64_certificates_only"]
    assert full.hexdigest() == digests["w64_full_stdout.txt"]


def test_w64_every_record_rechecked_on_the_device():
    eng = engine()
    c, recs = eng.run_window(*W64)
    assert c["rung"] == len(recs) == 8284620 and c["survivors"] == 0 and c["direct"] == 0
    assert np.all(recs["kind"] == es_sieve.ES_REC_RUNG)
    ok = np.ones(len(recs), dtype=bool)
    step = 1 << 21
    for a in range(0, len(recs), step):
        ok[a:a + step] = eng.check_records(recs[a:a + step])
    assert ok.all(), np.nonzero(~ok)[0][:10]
    # a planted mistake in one record is caught (the identity no longer holds)
    bad = recs[:4].copy()
    bad["c"][1] += 1
    assert eng.check_records(bad).tolist() == [True, False, True, True]
