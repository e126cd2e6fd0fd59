"""The drop-in binary itself on the GPU: rung_scan3_gb300 run as a subprocess exactly as a
caller of the reference's rung_scan3 runs it (sieve/rung_scan3.cpp:960-1163), gated the way the
reference gates its own scanner (tests/diff3.sh: byte-equal or set-equal stdout, SUMMARY equal,
--seg invariance, shard tiling) against the records the reference's own binaries produced.

Exit codes are part of the contract: 0 without survivors, 2 with survivors (the record is still
valid), 1 on every refusal (unknown flag, floor, ceiling, unreadable or empty filter file).
"""
import os
import subprocess

import pytest

import es_sieve
import workloads
from conftest import golden, read, split_stream, strip_for_cover_scan

pytestmark = pytest.mark.gpu

CLI = es_sieve.CLI_PATH
GPU = golden("filters", "f_M2042040_mmax2000_gpu.txt")
RT = golden("filters", "f_M2042040_mmax2000_runtime.txt")
C1 = golden("filters", "f_M120120_mmax2000_runtime.txt")
D3 = ["1000000000000", "1000200000000"]


def cli(*args, stdin=None):
    r = subprocess.run([CLI] + [str(a) for a in args], capture_output=True, text=True, timeout=600, input=stdin)
    return r.returncode, r.stdout, r.stderr


def expected_rc(text):
    """What rung_scan3 exits with for this record: 2 when a SUMMARY reports survivors."""
    return 2 if any(" survivors=0" not in ln for ln in split_stream(text)[1]) else 0


ROWS = [
    # (fixture under gen/, argv after the binary)
    ("c1_runtime.out", [workloads.c1()["lo"], workloads.c1()["hi"], "--wheel", 120120, "--filters", C1]),
    ("c1_default.out", [workloads.c1()["lo"], workloads.c1()["hi"], "--wheel", 120120]),
    ("d3_120120_m200.out", D3 + ["--wheel", 120120, "--mmax", 200]),
    ("d3_120120_m200.out", D3 + ["--wheel", 120120, "--mmax", 200, "--seg", 4096]),
    ("d3_120120_m200.out", D3 + ["--wheel", 120120, "--mmax", 200, "--threads", 3, "--progress", 5]),
    ("d3_120120_m200_sieve1000.out", D3 + ["--wheel", 120120, "--mmax", 200, "--sieve", 1000]),
    ("d3_120120_m2000.out", ["1000000000000", "1000010000000", "--wheel", 120120, "--mmax", 2000]),
    ("d3_2042040_m200.out", D3 + ["--wheel", 2042040, "--mmax", 200]),
    ("d3_2042040_m200_nosurv.out", D3 + ["--wheel", 2042040, "--mmax", 200, "--no-emit-survivors"]),
    ("c2_gpu.out", [workloads.c2()["lo"], workloads.c2()["hi"], "--filters", GPU]),
    ("c2_runtime.out", [workloads.c2()["lo"], workloads.c2()["hi"], "--filters", RT]),
    ("c3_gpu.out", [workloads.c3()["lo"], workloads.c3()["hi"], "--filters", GPU]),
    ("top_gpu_sieve500.out", [workloads.DIRECT_PMAX - (1 << 32), workloads.DIRECT_PMAX, "--filters", GPU,
                              "--sieve", 500]),
]


@pytest.mark.parametrize("name,args", ROWS, ids=["%s %s" % (n, " ".join(map(str, a[2:]))) for n, a in ROWS])
def test_cli_stdout_byte_identical_to_the_reference(name, args):
    want = read("gen", name)
    rc, out, err = cli(*args)
    assert out == want, err
    assert rc == expected_rc(want)


def test_cli_shards_tile_the_window():
    """--shard i/4 (ceil-span tiling, sieve/rung_scan3.cpp:1022-1027): each shard byte-equal to
    the reference's, and the four together carry the whole window's certificates and counts."""
    whole_certs, whole_sum = split_stream(read("gen", "d3_120120_m200.out"))
    certs, counts = [], {}
    for i in range(4):
        want = read("gen", "d3_120120_m200_shard%d_4.out" % i)
        rc, out, err = cli(*(D3 + ["--wheel", 120120, "--mmax", 200, "--shard", "%d/4" % i]))
        assert out == want, err
        assert rc == expected_rc(want)
        c, s = split_stream(out)
        certs += c
        for kv in s[0].split()[1:]:
            k, v = kv.split("=")
            if k in es_sieve.COUNTER_NAMES:
                counts[k] = counts.get(k, 0) + int(v)
    assert sorted(certs) == sorted(whole_certs)
    for kv in whole_sum[0].split()[1:]:
        k, v = kv.split("=")
        if k in es_sieve.COUNTER_NAMES:
            assert counts[k] == int(v), k


def test_cli_no_rung_hook_matches_cover_scan():
    """cover_scan's --no-rung test hook (sieve/cover_scan.cpp:395, :431): stage D skipped, every
    prime through the direct search; the same certificate set and counters as cover_scan."""
    want = read("gen", "d3_120120_m200_norung_cover_scan.out")
    rc, out, err = cli(*(D3 + ["--wheel", 120120, "--mmax", 200, "--no-rung"]))
    gc, gs = split_stream(out)
    wc, ws = split_stream(want)
    assert sorted(gc) == sorted(wc)
    assert [strip_for_cover_scan(x) for x in gs] == [strip_for_cover_scan(x) for x in ws]
    assert rc == expected_rc(want), err


def test_cli_batch_and_serve_modes():
    """--batch FILE and --serve FILE: each window's stream and SUMMARY in file order, byte-equal
    to the reference's sweep over the same windows; --serve also from standard input."""
    wf = golden("gen", "batch48.windows")
    want = read("gen", "batch48.out")
    for args, stdin in ((["--batch", wf], None), (["--serve", wf], None), (["--serve", "-"], open(wf).read())):
        rc, out, err = cli(*(args + ["--filters", GPU]), stdin=stdin)
        assert out == want, (args, err)
        assert rc == expected_rc(want)


def test_cli_refusals_exit_1(tmp_path):
    empty = tmp_path / "empty.txt"
    empty.write_text("# no filters here\n")
    cases = [
        (D3 + ["--bogus"], "unknown option"),
        ([workloads.DIRECT_PMAX - 10, workloads.DIRECT_PMAX + 1, "--filters", GPU], "stage-E ceiling"),
        ([255254, 300000, "--filters", GPU], "LO must exceed"),
        (D3 + ["--filters", str(tmp_path / "missing.txt")], "cannot open"),
        (D3 + ["--filters", str(empty)], "no FILTER lines"),
        (D3 + ["--order", "sideways"], "--order"),
    ]
    for args, msg in cases:
        rc, out, err = cli(*args)
        assert rc == 1 and msg in err and out == "", (args, rc, err)


def test_cli_verify_mode():
    rc, out, err = cli("--verify")
    assert rc == 0, out + err
    assert out.rstrip().endswith("SELF-TEST PASSED")
    assert "FAIL" not in out


@pytest.mark.parametrize("h", [9223372036854770000, 9223372036854775808, 9999999999999990000,
                               18446744065119000000])
def test_cli_check_direct_mode(h):
    """--check-direct LO N (sieve/rung_scan3.cpp:798-817): stage E on the first N primes at or
    above LO; stdout byte-equal to the reference's (Makefile:98-103 rows)."""
    rc, out, err = cli("--check-direct", h, 20)
    assert rc == 0, err
    assert out == read("gen", "direct_%d.out" % h)


def test_cli_check_factor_mode():
    """--check-factor (sieve/rung_scan3.cpp:459-530): the adversarial factorization battery on the
    device; every product of reported prime powers gives back n and every factor is prime."""
    rc, out, err = cli("--check-factor")
    assert rc == 0, out + err
    assert out.startswith("ok") and "bad products: 0, composite factors: 0" in out


def test_cli_round_order_stdout():
    """--order round: the production driver's order (rounds of --seg positions, lanes in wheel
    order within a round); with --seg 4096 the d3 window has several rounds per lane, so the
    stream is a different permutation of the same lines, and --order lane is rung_scan3's."""
    want = read("gen", "d3_2042040_m200.out")
    rc_l, lane, _ = cli(*(D3 + ["--wheel", 2042040, "--mmax", 200, "--order", "lane"]))
    assert lane == want
    rc_r, rnd, err = cli(*(D3 + ["--wheel", 2042040, "--mmax", 200, "--order", "round", "--seg", 16]))
    assert rc_r == rc_l == expected_rc(want), err
    lc, ls = split_stream(lane)
    rc_, rs = split_stream(rnd)
    assert rs == ls and sorted(rc_) == sorted(lc)
    assert rc_ != lc   # 16-position rounds over ~48 positions per lane reorder the lines
