"""The stage-D elliptic-curve method (erdos-strauss_gb300/csrc/es_ecm.cuh) on the CPU: its
constant tables against their definitions, and its arithmetic compiled for the host."""
import math
import os
import re
import shutil
import subprocess

import pytest

from conftest import PKG

HDR = os.path.join(PKG, "csrc", "es_ecm.cuh")


def _primes(n):
    s = bytearray([1]) * (n + 1)
    s[0] = s[1] = 0
    for i in range(2, int(n ** 0.5) + 1):
        if s[i]:
            s[i * i::i] = bytearray(len(s[i * i::i]))
    return [i for i in range(n + 1) if s[i]]


def _const(text, name):
    return int(re.search(r"constexpr (?:u32|int) %s = (\d+);" % name, text).group(1))


def _array(text, name):
    body = re.search(r"%s\[[^\]]*\] = \{([^}]*)\}" % name, text).group(1)
    return [int(x.strip().rstrip("u"), 0) for x in body.split(",") if x.strip()]


def test_tables_match_their_definitions():
    text = open(HDR).read()
    b1, b2, d = _const(text, "ECM_B1"), _const(text, "ECM_B2"), _const(text, "ECM_D")
    k = 1
    for p in _primes(b1):
        q = p
        while q * p <= b1:
            q *= p
        k *= q
    assert k == math.lcm(*range(1, b1 + 1))
    assert _const(text, "ECM_K_BITS") == k.bit_length()
    words = _array(text, "ECM_K")
    assert sum(w << (32 * i) for i, w in enumerate(words)) == k
    js = [j for j in range(1, d // 2, 2) if math.gcd(j, d) == 1]
    assert _array(text, "ECM_J") == js and _const(text, "ECM_NJ") == len(js)
    m1 = _const(text, "ECM_M1")
    assert m1 == (b2 + d // 2) // d
    ps = {p for p in _primes(b2) if p > b1}
    pairs = _array(text, "ECM_PAIRS")
    assert len(pairs) == m1
    covered = set()
    for m in range(1, m1 + 1):
        want = sum(1 << i for i, j in enumerate(js) if m * d + j in ps or m * d - j in ps)
        assert pairs[m - 1] == want, m
        covered |= {m * d + j for i, j in enumerate(js) if want >> i & 1}
        covered |= {m * d - j for i, j in enumerate(js) if want >> i & 1}
    assert ps <= covered


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_host_build_splits_hard_semiprimes(tmp_path):
    exe = str(tmp_path / "ecm_host_check")
    src = os.path.join(os.path.dirname(__file__), "ecm_host_check.cpp")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(PKG, "csrc"), src, "-o", exe], check=True)
    out = subprocess.run([exe, "40"], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    rates = {int(m.group(1)): (float(m.group(2)), float(m.group(3)))
             for m in re.finditer(r"bits (\d+) curves ([\d.]+) warps ([\d.]+)", out.stdout)}
    assert sorted(rates) == list(range(18, 32))
    # the per-curve rate falls with the size of the smaller prime (B1 = 40, B2 = 2000: about
    # 0.65 at 18 bits, 0.15 at 24, 0.02 at 31); one round of 32 curves splits every pair with
    # a prime below 2^22 and about half of the 31-bit pairs
    assert all(rates[b][1] == 1.0 for b in range(18, 23)), rates
    assert rates[18][0] > 0.5 and 0.08 < rates[24][0] < 0.25 and 0.003 < rates[31][0] < 0.05, rates
    assert rates[31][1] > 0.1, rates
