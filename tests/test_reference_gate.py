"""The host certificate gate oracle/verify.py against the reference's own gate.

oracle/verify.py restates sieve/verify_covers.py:246-275 (verify_output: exact rational
re-derivation of every RUNG and SOLVED line); the GPU tests use the restatement because the
reference tree is absent on the GPU host. Here, where the tree is present, both gates read the
same fixture files -- the reference's own records, a planted-mistake file, survivors -- and must
reach the same verdicts and counts. Skipped where there is no reference tree.
"""
import os
import re
import subprocess
import sys

import pytest

from conftest import ROOT, golden, read

sys.path.insert(0, ROOT)
import __graft_entry__  # noqa: E402
import verify  # noqa: E402

REF = __graft_entry__.reference_tree()
pytestmark = pytest.mark.skipif(REF is None, reason="no reference tree on this host")

FILES = ["gen/c1_runtime.out", "gen/c2_gpu.out", "gen/c3_gpu.out", "gen/d3_120120_m200_norung_cover_scan.out",
         "gen/direct_18446744065119000000.out", "gen/batch48.out", "decades/d19.txt",
         "windows/w19_certificates.txt", "windows/w64_head.txt", "windows/w64_tail.txt"]


def reference_gate(path):
    r = subprocess.run([sys.executable, os.path.join(REF, "sieve", "verify_covers.py"), path],
                       capture_output=True, text=True, timeout=600)
    m = re.search(r"verified: (\d+) RUNG, (\d+) SOLVED; (\d+) bad, (\d+) survivors", r.stdout)
    assert m, r.stdout[-2000:] + r.stderr[-2000:]
    return tuple(int(x) for x in m.groups()), r.returncode


@pytest.mark.parametrize("name", FILES)
def test_same_verdicts_as_the_reference_gate(name):
    path = golden(*name.split("/"))
    ref, rc = reference_gate(path)
    mine = verify.check_text(read(*name.split("/")))
    assert mine == ref
    assert rc == (1 if ref[2] or ref[3] else 0)


def test_both_gates_reject_the_same_planted_mistakes(tmp_path):
    lines = read("gen", "c2_gpu.out").splitlines(keepends=True)
    certs = [ln for ln in lines if ln.startswith(("RUNG", "SOLVED"))]
    bad = list(certs)
    t = bad[0].split()
    t[4] = str(int(t[4]) + 1)                          # u off by one
    bad[0] = " ".join(t) + "\n"
    t = bad[1].split()
    t[3] = "7" if t[3] != "7" else "3"                 # another rung
    bad[1] = " ".join(t) + "\n"
    direct = read("gen", "direct_9223372036854775808.out").splitlines(keepends=True)
    t = direct[0].split()
    t[5] = str(int(t[5]) + 1)                          # SOLVED k off by one
    bad.append(" ".join(t) + "\n")
    bad.append("SURVIVOR 18446744065119614899\n")
    f = tmp_path / "planted.txt"
    f.write_text("".join(bad))
    ref, rc = reference_gate(str(f))
    assert verify.check_text("".join(bad)) == ref
    assert ref[2] == 3 and ref[3] == 1 and rc == 1
