"""GPU parity: the engine through its C ABI against the reference's golden records and the
CPU oracle. Integer results, so every comparison is exact (byte-identical text, equal sets,
equal counters)."""
import os

import numpy as np
import pytest

import es_sieve
import oracle
import workloads
from conftest import golden, read, split_stream, strip_for_cover_scan

pytestmark = pytest.mark.gpu

GPU_TABLE = "f_M2042040_mmax2000_gpu.txt"
RT_TABLE = "f_M2042040_mmax2000_runtime.txt"
C1_TABLE = "f_M120120_mmax2000_runtime.txt"

_engines = {}


def engine(wheel=2042040, table=GPU_TABLE, mmax=10000, sieve_p=0, no_rung=False):
    key = (wheel, table, mmax, sieve_p, no_rung)
    if key not in _engines:
        f = es_sieve.load_filters(golden("filters", table)) if table else None
        _engines[key] = es_sieve.Engine(wheel=wheel, filters=f, mmax=mmax, sieve_p=sieve_p, no_rung=no_rung)
    return _engines[key]


def test_c1_runtime_table_byte_identical():
    c = workloads.c1()
    assert engine(120120, C1_TABLE).stream(c["lo"], c["hi"]) == read("gen", "c1_runtime.out")


def test_c1_default_set_byte_identical_and_matches_cover_scan():
    c = workloads.c1()
    got = engine(120120, None).stream(c["lo"], c["hi"])
    assert got == read("gen", "c1_default.out")
    cov = read("gen", "c1_default_cover_scan.out")
    assert strip_for_cover_scan(split_stream(got)[1][0]) == strip_for_cover_scan(split_stream(cov)[1][0])


@pytest.mark.parametrize("name,table", [("c2_gpu", GPU_TABLE), ("c2_runtime", RT_TABLE), ("c3_gpu", GPU_TABLE)])
def test_2p34_windows_byte_identical(name, table):
    c = workloads.c2() if name.startswith("c2") else workloads.c3()
    assert engine(2042040, table).stream(c["lo"], c["hi"]) == read("gen", name + ".out")


@pytest.mark.parametrize("k", list(range(6, 20)))
def test_decade_windows(k):
    """data/rederive/decades/d<k>.txt: SUMMARY byte-equal, certificate set equal (the
    fixture's stream is round-major, so compare sorted)."""
    ref = read("decades", "d%d.txt" % k)
    certs, summ = split_stream(ref)
    lo = int(summ[0].split("lo=")[1].split()[0])
    hi = int(summ[0].split("hi=")[1].split()[0])
    got = engine().stream(lo, hi)
    gc, gs = split_stream(got)
    assert gs == summ
    assert sorted(gc) == sorted(certs)


def test_w19_window_complete_certificate_set():
    ref = read("windows", "w19_certificates.txt")
    certs, summ = split_stream(ref)
    got = engine().stream(5000000000000000000, 5000001000000000000)
    gc, gs = split_stream(got)
    assert gs == summ
    assert sorted(gc) == sorted(certs)
    assert len(gc) == 8413


@pytest.mark.parametrize("name,args", [
    ("d3_120120_m200", dict(wheel=120120, table=None, mmax=200)),
    ("d3_120120_m200_sieve1000", dict(wheel=120120, table=None, mmax=200, sieve_p=1000)),
    ("d3_2042040_m200", dict(wheel=2042040, table=None, mmax=200)),
])
def test_differential_gate_rows(name, args):
    lo, hi = 1000000000000, 1000200000000
    assert engine(**args).stream(lo, hi) == read("gen", name + ".out")


def test_differential_gate_m2000():
    assert engine(120120, None, mmax=2000).stream(1000000000000, 1000010000000) == read("gen", "d3_120120_m2000.out")


def test_no_emit_survivors_and_cover_scan_agreement():
    lo, hi = 1000000000000, 1000200000000
    e = engine(2042040, None, mmax=200)
    assert e.stream(lo, hi, emit_survivors=False) == read("gen", "d3_2042040_m200_nosurv.out")
    got = engine(120120, None, mmax=200).stream(lo, hi)
    cov = read("gen", "d3_120120_m200_cover_scan.out")
    gc, gs = split_stream(got)
    cc, cs = split_stream(cov)
    assert sorted(gc) == sorted(cc)
    assert strip_for_cover_scan(gs[0]) == strip_for_cover_scan(cs[0])


def test_shards_tile_the_range():
    lo, hi = 1000000000000, 1000200000000
    e = engine(120120, None, mmax=200)
    for i in range(4):
        a, b = workloads.shard_bounds(lo, hi, i, 4)
        assert e.stream(a, b) == read("gen", "d3_120120_m200_shard%d_4.out" % i)


def test_stage_e_inside_a_scan_matches_cover_scan_no_rung():
    lo, hi = 1000000000000, 1000200000000
    got = engine(120120, None, mmax=200, no_rung=True).stream(lo, hi)
    ref = read("gen", "d3_120120_m200_norung_cover_scan.out")
    gc, gs = split_stream(got)
    rc, rs = split_stream(ref)
    assert sorted(gc) == sorted(rc)
    assert strip_for_cover_scan(gs[0]) == strip_for_cover_scan(rs[0])


def test_top_of_range_with_stage_b_prime():
    top = workloads.DIRECT_PMAX
    got = engine(2042040, GPU_TABLE, sieve_p=500).stream(top - (1 << 32), top)
    assert got == read("gen", "top_gpu_sieve500.out")


def _batch48():
    wins = [tuple(int(x) for x in ln.split()) for ln in read("gen", "batch48.windows").splitlines()]
    blocks, cur = [], []
    for ln in read("gen", "batch48.out").splitlines(keepends=True):
        cur.append(ln)
        if ln.startswith("SUMMARY "):
            blocks.append("".join(cur))
            cur = []
    return wins, blocks


@pytest.mark.parametrize("schedule", [es_sieve.ES_SCHED_PERSISTENT, es_sieve.ES_SCHED_PLAIN])
def test_batch_sample_per_window_records(schedule):
    wins, blocks = _batch48()
    e = engine()
    per, recs = e.run_batch(wins, schedule=schedule)
    for i, (lo, hi) in enumerate(wins):
        mine = recs[recs["window"] == i]
        assert e.text(lo, hi, per[i], mine) == blocks[i], "window %d" % i


def test_batch_equals_windows_run_alone():
    wins, blocks = _batch48()
    e = engine()
    for i in (0, 5, 17, 47):
        assert e.stream(*wins[i]) == blocks[i]


def test_many_primes_warp_and_block_phases():
    """A 10^12-integer window at 10^17 has about 9 K primes, more than the stage-D grid has
    warps: most take the warp-per-prime phase and the last ones the block phase. The
    records must equal those of the same window cut into pieces small enough that all their
    primes go to the block phase."""
    e = engine()
    lo, hi = 10 ** 17 + 99991, 10 ** 17 + 99991 + 10 ** 12
    c, r = e.run_window(lo, hi)
    assert c["rung"] > 8000
    step = (hi - lo) // 8
    got, n_rung = [], 0
    for i in range(8):
        a, b = lo + i * step, (lo + (i + 1) * step if i < 7 else hi)
        pc, pr = e.run_window(a, b)                 # about 1.1 K primes each: block phase only
        n_rung += pc["rung"]
        got += [(int(x["p"]), int(x["a"]), int(x["b"]), int(x["c"]), int(x["d"])) for x in pr]
    assert n_rung == c["rung"]
    assert sorted(got) == sorted((int(x["p"]), int(x["a"]), int(x["b"]), int(x["c"]), int(x["d"])) for x in r)


def test_repeat_runs_are_identical():
    c = workloads.c3()
    e = engine()
    assert e.stream(c["lo"], c["hi"]) == e.stream(c["lo"], c["hi"])


def test_refusals_and_empty_window():
    e = engine()
    with pytest.raises(es_sieve.EsError) as ex:
        e.run_window(255254, 10 ** 9)
    assert ex.value.status == es_sieve.ES_ERR_RANGE
    with pytest.raises(es_sieve.EsError) as ex:
        e.run_window(10 ** 18, workloads.DIRECT_PMAX + 1)
    assert ex.value.status == es_sieve.ES_ERR_RANGE
    c, r = e.run_window(10 ** 12, 10 ** 12)
    assert all(v == 0 for v in c.values()) and len(r) == 0
    c, r = e.run_window(10 ** 12, 10 ** 12 + 1)     # one integer, not in any lane
    assert c["positions"] == 0


# ------------------------------------------------------------------ device probes vs oracle
@pytest.mark.parametrize("base", [10 ** 6, 2 ** 32 - 5000, 10 ** 12, 2 ** 62, 2 ** 63 - 2000, 2 ** 64 - 60000])
def test_primality_dense_ranges(base):
    ns = np.arange(base, base + 40000, dtype=np.uint64) if base + 40000 < 2 ** 64 else \
        np.arange(base, 2 ** 64 - 1, dtype=np.uint64)
    got = engine().is_prime(ns)
    want = [oracle.is_prime(int(n)) for n in ns]
    assert list(got) == want


def _battery(seed=7, n=300):
    g = workloads.SplitMix64(seed)
    vals = []
    for dec in [10 ** k for k in range(6, 19)]:
        vals += [dec + g.next() % (9 * dec) for _ in range(n // 10)]
    def nextp(a):
        while not oracle.is_prime(a):
            a += 1
        return a
    for _ in range(n // 5):   # hard semiprimes both sides of 2^63
        a = nextp(3037000000 + g.next() % 1257000000)
        b = nextp(2147483648 + g.next() % 2147000000)
        if a * b <= workloads.DIRECT_PMAX + 2049:
            vals.append(a * b)
        c = nextp(2147483648 + g.next() % 2147000000)
        vals.append(c * c)
    for _ in range(n // 5):   # three large prime factors
        a, b = nextp(65537 + g.next() % 200000), nextp(65537 + g.next() % 2000000)
        c = nextp(65537 + g.next() % ((2 ** 64 - 1) // (a * b) - 65537))
        if a * b * c < 2 ** 64:
            vals.append(a * b * c)
    B = 65536 * 65536
    vals += [B - 1, B, B + 1, 2 ** 63 - 1, 2 ** 63, 2 ** 63 + 1, 2 ** 64 - 1, 18446744065119617025, 1, 2, 3, 4]
    return vals


def test_factorization_battery():
    vals = _battery()
    got = engine().factor(vals)
    for v, f in zip(vals, got):
        assert f == oracle.factor(v), v


def test_factorization_ecm_range():
    """Cofactors below 2^62 go through rho and then the lazy-arithmetic ECM rounds, those from
    2^62 up through exact rho: balanced semiprimes of 20-31-bit primes, pairs straddling the
    2^62 switch, and three-prime products, against the oracle's factorization."""
    g = workloads.SplitMix64(62)
    def nextp(a):
        while not oracle.is_prime(a):
            a += 1
        return a
    vals = []
    for bits in range(20, 32):
        for _ in range(6):
            a = nextp((1 << (bits - 1)) + g.next() % (1 << (bits - 1)))
            b = nextp((1 << (61 - bits)) + g.next() % (1 << (61 - bits)))
            vals.append(a * b)
    for _ in range(12):                                  # around 2^62
        a = nextp(2147483648 + g.next() % 2147483648)
        b = nextp((1 << 62) // a - 2000 + g.next() % 4000)
        vals.append(a * b)
    for _ in range(12):
        a, b = nextp(65537 + g.next() % 1000000), nextp(65537 + g.next() % 1000000)
        c = nextp(65537 + g.next() % ((1 << 62) // (a * b) - 65537))
        vals.append(a * b * c)
    assert any(v < 1 << 62 for v in vals) and any(v >= 1 << 62 for v in vals)
    got = engine().factor(vals)
    for v, f in zip(vals, got):
        assert f == oracle.factor(v), v


def _primes_at(height, count):
    out, p = [], height | 1
    while len(out) < count:
        if oracle.is_prime(p):
            out.append(p)
        p += 2
    return out


@pytest.mark.parametrize("height", [10 ** 7, 10 ** 12, 10 ** 16, 5 * 10 ** 18, 17 * 10 ** 18, workloads.DIRECT_PMAX - 10 ** 9])
def test_solve_rung_vs_oracle(height):
    ps = _primes_at(height, 200)
    got = engine().solve_rung(ps)
    for p, g in zip(ps, got):
        want = oracle.solve_rung(p)
        assert g == want, p


@pytest.mark.parametrize("h", [9223372036854770000, 9223372036854775808, 9999999999999990000, 18446744065119000000])
def test_solve_direct_check_direct_rows(h):
    ref = read("gen", "direct_%d.out" % h).splitlines(keepends=True)
    ps = [int(ln.split()[1]) for ln in ref]
    assert engine().solve_direct(ps) == ref


def test_solve_direct_vs_oracle_small():
    ps = _primes_at(10 ** 9, 100) + _primes_at(10 ** 17, 50)
    got = engine().solve_direct(ps)
    assert got == [oracle.solve_direct(p) for p in ps]


def test_every_emitted_certificate_rechecks_in_exact_arithmetic():
    """The reference's exact-rational gate (sieve/verify_covers.py), restated in
    oracle/verify.py, over everything the engine emits for a spread of windows."""
    import verify
    total = 0
    cases = [(engine(), workloads.c3()["lo"], workloads.c3()["hi"]),
             (engine(), 5000000000000000000, 5000001000000000000),
             (engine(120120, None, mmax=200, no_rung=True), 1000000000000, 1000200000000),
             (engine(2042040, GPU_TABLE, sieve_p=500), workloads.DIRECT_PMAX - (1 << 32), workloads.DIRECT_PMAX)]
    for e, lo, hi in cases:
        r, s_, bad, surv = verify.check_text(e.stream(lo, hi))
        assert bad == 0 and surv == 0
        total += r + s_
    wins, _ = _batch48()
    per, recs = engine().run_batch(wins)
    for i, (lo, hi) in enumerate(wins):
        r, s_, bad, surv = verify.check_text(engine().text(lo, hi, per[i], recs[recs["window"] == i]))
        assert bad == 0 and surv == 0
        total += r + s_
    assert total > 9000


def _records_from_text(text):
    recs = []
    for ln in text.splitlines():
        t = ln.split()
        if not t or t[0] == "SUMMARY":
            continue
        if t[0] == "RUNG":
            p, A, r, u = map(int, t[1:5])
            recs.append((es_sieve.ES_REC_RUNG, 0, 0, 0, 0, p, A, r, u & (2 ** 64 - 1), u >> 64))
        elif t[0] == "SOLVED":
            p, a, c, d, k = map(int, t[1:6])
            recs.append((es_sieve.ES_REC_SOLVED, 0, 0, 0, 0, p, a, c, d, k))
        elif t[0] == "SURVIVOR":
            recs.append((es_sieve.ES_REC_SURVIVOR, 0, 0, 0, 0, int(t[1]), 0, 0, 0, 0))
    return np.array(recs, dtype=es_sieve.RECORD_DTYPE)


def test_device_certificate_check_on_reference_records_and_planted_mistakes():
    """es_check_records re-derives each identity on the device: every certificate the
    reference emitted (w19, c3, cover_scan's stage-E rows) passes; copies with one field
    changed (planted here, on the CPU) and SURVIVOR lines fail."""
    good = np.concatenate([_records_from_text(read("windows", "w19_certificates.txt")),
                           _records_from_text(read("gen", "c3_gpu.out")),
                           _records_from_text(read("gen", "d3_120120_m200_norung_cover_scan.out"))])
    assert (good["kind"] == es_sieve.ES_REC_SOLVED).sum() > 0 and len(good) > 8500
    assert engine().check_records(good).all()
    bad = []
    for field in ("a", "b", "c", "d"):
        x = good[:64].copy()
        x[field] += 1
        bad.append(x)
    x = good[:8].copy()
    x["p"] += 2
    bad.append(x)
    bad = np.concatenate(bad)
    assert not engine().check_records(bad).any()
    s = good[:4].copy()
    s["kind"] = es_sieve.ES_REC_SURVIVOR
    assert not engine().check_records(s).any()


def test_cli_serve_streams_each_window_in_input_order(tmp_path):
    """rung_scan3_gb300 --serve -: windows read from stdin are submitted as they arrive and
    printed in input order; the output is the batch sample's golden record."""
    import subprocess
    wins = [tuple(int(x) for x in ln.split()) for ln in read("gen", "batch48.windows").splitlines()]
    stdin = "".join("%d %d\n" % w for w in wins)
    r = subprocess.run([es_sieve.CLI_PATH, "--serve", "-", "--filters", golden("filters", GPU_TABLE)],
                       input=stdin, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-500:]
    assert r.stdout == read("gen", "batch48.out")


def test_device_failure_surfaces_as_status_and_engine_stays_usable():
    """With the test hook that cuts Brent's rho to 64 steps, a semiprime of two 31-bit primes
    cannot be split: the probe and a window that needs it fail with ES_ERR_DEVICE_STATUS
    ("rho-budget"), nothing wrong is emitted, and the same engine keeps working."""
    e = es_sieve.Engine(wheel=2042040, filters=golden("filters", GPU_TABLE), test_rho_budget=True)
    try:
        semi = 2147483659 * 2147483693
        with pytest.raises(es_sieve.EsError) as ex:
            e.factor([semi])
        assert ex.value.status == es_sieve.ES_ERR_DEVICE_STATUS and "rho-budget" in str(ex.value)
        assert e.factor([2 ** 40 * 3 ** 5]) == [oracle.factor(2 ** 40 * 3 ** 5)]
        c = workloads.c3()
        with pytest.raises(es_sieve.EsError) as ex:
            e.run_window(c["lo"], c["hi"])
        assert ex.value.status == es_sieve.ES_ERR_DEVICE_STATUS
        assert list(e.is_prime([2 ** 61 - 1, 2 ** 61 + 1])) == [True, False]
    finally:
        e.close()
    assert engine().stream(workloads.c3()["lo"], workloads.c3()["hi"]) == read("gen", "c3_gpu.out")
