"""The CPU oracle pinned against the reference's golden vectors (no GPU needed).

The oracle is the checker of every GPU parity test, so it is itself checked first: against
the records the reference ships (data/rederive/decades, the w19 window, the class tables,
the self-test constants) and against the reference scanners' own output on the seeded
configurations (tests/golden/gen, made by tests/golden/make_fixtures.py).
"""
import hashlib
import os
import subprocess

import pytest

import oracle
import workloads
from conftest import golden, read, split_stream, strip_for_cover_scan

CLI = oracle.CLI


@pytest.fixture(scope="module", autouse=True)
def built():
    oracle.build()


def run(*args):
    r = subprocess.run([CLI] + [str(a) for a in args], capture_output=True, text=True, timeout=600)
    return r.returncode, r.stdout


def test_self_test_constants():
    rc, out = run("--verify")
    assert rc == 0 and "SELF-TEST PASSED" in out
    assert "FAIL" not in out


def test_class_tables_match_published_digests():
    want = dict(ln.split()[::-1] for ln in read("class_tables.sha256").splitlines())
    for M in (120120, 2042040):
        rc, out = run("--dump-classes", "--wheel", M)
        assert rc == 0
        assert hashlib.sha256(out.encode()).hexdigest() == want["class_table_%d.txt" % M]


def test_wheel_constants():
    w = oracle.wheel(2042040)
    assert len(w["classes"]) == 2308 and w["max_pmin"] == 255254 and w["fnv64"] == 0xb9b5d1408da3428e
    w = oracle.wheel(120120)
    assert len(w["classes"]) == 220 and w["max_pmin"] == 15014 and w["n_f1_only"] == 920


@pytest.mark.parametrize("name,args", [
    ("c1_runtime", lambda F: [10 ** 9, 10 ** 9 + 2 ** 26, "--wheel", 120120, "--filters", F("f_M120120_mmax2000_runtime.txt")]),
    ("c1_default", lambda F: [10 ** 9, 10 ** 9 + 2 ** 26, "--wheel", 120120]),
    ("d3_120120_m200", lambda F: [10 ** 12, 1000200000000, "--wheel", 120120, "--mmax", 200]),
    ("d3_120120_m200_sieve1000", lambda F: [10 ** 12, 1000200000000, "--wheel", 120120, "--mmax", 200, "--sieve", 1000]),
    ("d3_120120_m2000", lambda F: [10 ** 12, 1000010000000, "--wheel", 120120, "--mmax", 2000]),
    ("d3_2042040_m200", lambda F: [10 ** 12, 1000200000000, "--wheel", 2042040, "--mmax", 200]),
    ("d3_2042040_m200_nosurv", lambda F: [10 ** 12, 1000200000000, "--wheel", 2042040, "--mmax", 200, "--no-emit-survivors"]),
    ("d3_120120_m200_shard2_4", lambda F: [10 ** 12, 1000200000000, "--wheel", 120120, "--mmax", 200, "--shard", "2/4"]),
])
def test_cli_byte_identical_to_reference(name, args):
    rc, out = run(*args(lambda f: golden("filters", f)))
    assert rc == 0
    assert out == read("gen", name + ".out")


@pytest.mark.parametrize("name", ["c2_gpu", "c2_runtime", "c3_gpu"])
def test_seeded_2p34_windows(name):
    c = workloads.c2() if name.startswith("c2") else workloads.c3()
    table = "f_M2042040_mmax2000_runtime.txt" if "runtime" in name else "f_M2042040_mmax2000_gpu.txt"
    rc, out = run(c["lo"], c["hi"], "--filters", golden("filters", table))
    assert out == read("gen", name + ".out")


def test_top_of_range_with_sieve():
    top = workloads.DIRECT_PMAX
    rc, out = run(top - 2 ** 32, top, "--filters", golden("filters", "f_M2042040_mmax2000_gpu.txt"), "--sieve", 500)
    assert out == read("gen", "top_gpu_sieve500.out")


@pytest.mark.parametrize("k", [6, 7, 8, 10, 13, 16, 19])
def test_decade_windows(k):
    certs, summ = split_stream(read("decades", "d%d.txt" % k))
    lo = int(summ[0].split("lo=")[1].split()[0])
    hi = int(summ[0].split("hi=")[1].split()[0])
    rc, out = run(lo, hi, "--filters", golden("filters", "f_M2042040_mmax2000_gpu.txt"))
    gc, gs = split_stream(out)
    assert gs == summ and sorted(gc) == sorted(certs)


def test_w19_window():
    certs, summ = split_stream(read("windows", "w19_certificates.txt"))
    rc, out = run(5000000000000000000, 5000001000000000000, "--filters", golden("filters", "f_M2042040_mmax2000_gpu.txt"))
    gc, gs = split_stream(out)
    assert gs == summ and sorted(gc) == sorted(certs)


def test_cover_scan_agreement_default_set():
    rc, out = run(10 ** 12, 1000200000000, "--wheel", 120120, "--mmax", 200)
    cov = read("gen", "d3_120120_m200_cover_scan.out")
    assert sorted(split_stream(out)[0]) == sorted(split_stream(cov)[0])
    assert strip_for_cover_scan(split_stream(out)[1][0]) == strip_for_cover_scan(split_stream(cov)[1][0])


@pytest.mark.parametrize("h", [9223372036854770000, 9223372036854775808, 9999999999999990000, 18446744065119000000])
def test_check_direct_rows(h):
    rc, out = run("--check-direct", h, 20)
    assert rc == 0 and out == read("gen", "direct_%d.out" % h)


def test_batch_sample_windows():
    wins = [tuple(int(x) for x in ln.split()) for ln in read("gen", "batch48.windows").splitlines()][:12]
    ref = read("gen", "batch48.out").splitlines(keepends=True)
    blocks, cur = [], []
    for ln in ref:
        cur.append(ln)
        if ln.startswith("SUMMARY "):
            blocks.append("".join(cur)); cur = []
    for (lo, hi), want in zip(wins, blocks):
        rc, out = run(lo, hi, "--filters", golden("filters", "f_M2042040_mmax2000_gpu.txt"))
        assert out == want


def test_refusals():
    assert run(255254, 10 ** 9)[0] == 1                        # LO at the floor
    assert run(10 ** 18, workloads.DIRECT_PMAX + 1)[0] == 1    # HI above the ceiling
    assert run(10 ** 12, 10 ** 13, "--bogus")[0] == 1          # unknown flag
    assert run(10 ** 12, 10 ** 13, "--filters", "/nonexistent")[0] == 1


def test_oracle_library_agrees_with_cli():
    mods, ress, ncov = oracle.default_filters(120120, 200)
    text, cnt = oracle.scan(10 ** 12, 1000200000000, 120120, mods, ress, ncov)
    ref = read("gen", "d3_120120_m200.out")
    assert ref.startswith(text)
    assert "positions=%d covered=%d" % (cnt["positions"], cnt["covered"]) in ref


def test_manifest_hashes():
    for ln in read("MANIFEST.txt").splitlines():
        if ln.startswith("#"):
            continue
        name, digest = ln.split()[:2]
        assert hashlib.sha256(open(golden(name), "rb").read()).hexdigest() == digest, name


@pytest.mark.skipif(not oracle.ref_binary("rung_scan3"), reason="reference scanners not built here")
def test_reference_binaries_regenerate_fixtures():
    """Where the reference tree is present, its scanners reproduce the committed fixtures."""
    r = subprocess.run([oracle.ref_binary("rung_scan3"), "1000000000", "1067108864", "--wheel", "120120",
                        "--filters", golden("filters", "f_M120120_mmax2000_runtime.txt")],
                       capture_output=True, text=True)
    assert r.stdout == read("gen", "c1_runtime.out")


def test_certificate_checker_on_reference_records():
    """The exact re-check accepts every certificate the reference emitted and rejects a
    planted mistake (planted here, on the CPU, in a copy of a line)."""
    import verify
    for name in ("windows/w19_certificates.txt", "gen/d3_120120_m200_norung_cover_scan.out", "gen/c3_gpu.out"):
        r, s_, bad, surv = verify.check_text(read(*name.split("/")))
        assert bad == 0 and surv == 0 and r + s_ > 0
    line = read("gen", "c3_gpu.out").splitlines()[0].split()
    line[4] = str(int(line[4]) + 1)                       # a wrong witness u
    assert verify.check_line(" ".join(line)) == ("RUNG", False)
    sl = read("gen", "d3_120120_m200_norung_cover_scan.out").splitlines()[0].split()
    sl[5] = str(int(sl[5]) + 1)                           # a wrong k
    assert verify.check_line(" ".join(sl)) == ("SOLVED", False)
