"""The GB300-tuned filter table (erdos-strauss_gb300/filter_tune.py), on the CPU.

* every filter of the shipped table is certified: an F1 cover of the oracle's generated set
  (m <= 2000, m not dividing M) or an F2 uniform rung certificate checked from its definition;
* the tuner's candidates include every filter of the reference's own gpu table, and its wheel
  lanes are the engine's class table;
* the shipped table is what the tuner writes from the committed GPU calibration.
The table's results on the device are pinned against the reference's scanner run on it in
tests/test_gpu_gb300_table.py."""
import hashlib
import os
import subprocess
import sys
from math import gcd

import pytest

import oracle
from conftest import PKG, golden

M = 2042040
TABLE = os.path.join(PKG, "tables", "f_M2042040_mmax2000_gb300.txt")
CAL = os.path.join(PKG, "tables", "calibration_batch4096.json")


def table_rows(path):
    return [(int(t[1]), int(t[2]), t[3]) for t in (ln.split() for ln in open(path)) if t and t[0] == "FILTER"]


def f2_certified(L, res):
    """Some coprime r <= 63, u <= 64 with L = 4ru certifies the class res (mod L): p = -r (mod 4),
    and q = p (p + r) / 4 satisfies u | q^2 and q = -u (mod r) (q mod ru depends on p mod L only)."""
    if L % 4:
        return False
    for r in range(1, 64):
        if (L // 4) % r:
            continue
        u = L // 4 // r
        if u > 64 or gcd(r, u) != 1 or (res + r) % 4:
            continue
        q = res * ((res + r) // 4)
        if (q * q) % u == 0 and (q + u) % r == 0:
            return True
    return False


def test_every_filter_of_the_tuned_table_is_certified():
    rows = table_rows(TABLE)
    assert len(rows) == len(set((m, r) for m, r, _ in rows)) > 3745
    mods, ress, _ = oracle.default_filters(M, mmax=2000)
    f1 = set(zip((int(m) for m in mods), (int(r) for r in ress)))
    for mod, res, fam in rows:
        assert M % mod != 0, (mod, res)
        if fam == "F1":
            assert (mod, res) in f1, (mod, res)
        else:
            assert fam == "F2" and f2_certified(mod, res), (mod, res)


def test_table_digest_matches_its_body():
    text = open(TABLE).read()
    body = "".join(ln for ln in text.splitlines(keepends=True) if ln.startswith("FILTER "))
    head = [ln for ln in text.splitlines() if ln.startswith("# sha256=")]
    assert head and head[0].split()[1] == "sha256=" + hashlib.sha256(body.encode()).hexdigest()


def test_candidates_cover_the_reference_table_and_lanes_are_the_wheel():
    sys.path.insert(0, PKG)
    import filter_tune
    cands = set((m, r) for m, r, _ in filter_tune.candidates(2000, M))
    ref = table_rows(golden("filters", "f_M2042040_mmax2000_gpu.txt"))
    assert all((m, r) in cands for m, r, _ in ref)
    import es_sieve
    cli = os.path.join(PKG, "rung_scan3_gb300")
    if not os.path.exists(cli):
        pytest.skip("command line not built")
    out = subprocess.run([cli, "--dump-classes", "--wheel", str(M)], capture_output=True, text=True).stdout
    classes = [int(ln.split()[1]) for ln in out.splitlines() if ln.startswith("CLASS ")]
    assert classes == list(filter_tune.wheel_lanes(M))
    del es_sieve


def test_shipped_table_is_the_tuners_choice(tmp_path):
    out = tmp_path / "t.txt"
    r = subprocess.run([sys.executable, os.path.join(PKG, "filter_tune.py"), "--calibrate", CAL, "--write", str(out)],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    assert out.read_text() == open(TABLE).read()
