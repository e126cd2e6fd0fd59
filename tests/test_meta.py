"""Shard records (run19 metas): the digest, the parser, the two emission orders, and the
reference's own production records re-derived on the GPU.

CPU: SHA-256 of the library against hashlib; the meta parser on a production meta
(data/c19/shard_0.meta); the audit; the round-order rearrangement, which turns the oracle's
lane-major text for the w19 window into the production driver's stream for it byte for byte.
GPU: the CLI's --meta reproduces that stream's digest, and in both orders matches digests
recomputed here from the engine's lane-major text."""
import ctypes as C
import hashlib
import os

import pytest

import es_sieve
import shard_meta
from conftest import golden, read

GPU_TABLE = golden("filters", "f_M2042040_mmax2000_gpu.txt")
M = 2042040


def _lib():
    lib = C.CDLL(es_sieve.LIB_PATH)
    lib.es_sha256_hex.restype = C.c_size_t
    lib.es_sha256_hex.argtypes = [C.c_void_p, C.c_size_t, C.c_char_p, C.c_size_t]
    return lib


def test_sha256_matches_hashlib():
    lib = _lib()
    for n in (0, 1, 3, 55, 56, 57, 63, 64, 65, 119, 120, 121, 1000, 65536, 100003):
        data = os.urandom(n)
        out = C.create_string_buffer(65)
        assert lib.es_sha256_hex(data, n, out, 65) == 64
        assert out.value.decode() == hashlib.sha256(data).hexdigest(), n
    out = C.create_string_buffer(64)
    assert lib.es_sha256_hex(b"x", 1, out, 64) == 0            # no room for the NUL


def test_sha256_builtin_backend_matches_hashlib():
    """The built-in SHA-256 (used when libcrypto is absent) gives the same digests."""
    import subprocess
    import sys
    code = ("import ctypes as C, hashlib, os, sys\n"
            "lib = C.CDLL(sys.argv[1])\n"
            "lib.es_sha256_hex.restype = C.c_size_t\n"
            "lib.es_sha256_hex.argtypes = [C.c_void_p, C.c_size_t, C.c_char_p, C.c_size_t]\n"
            "for n in (0, 1, 55, 56, 63, 64, 65, 119, 120, 4096, 100003, 1 << 20):\n"
            "    d = os.urandom(n); out = C.create_string_buffer(65)\n"
            "    lib.es_sha256_hex(d, n, out, 65)\n"
            "    assert out.value.decode() == hashlib.sha256(d).hexdigest(), n\n"
            "print('ok')\n")
    env = dict(os.environ, ES_SHA256_BUILTIN="1")
    r = subprocess.run([sys.executable, "-c", code, es_sieve.LIB_PATH], env=env, capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stderr


def test_parse_production_meta():
    d = shard_meta.parse_meta(read("metas", "c19_shard_0.meta"))
    assert d["complete"] and d["idx"] == 0 and d["nshards"] == 250 and d["rc"] == 0
    assert d["certs"] == 394469504 == d["rung"] + d["direct"]
    assert d["cert_sha256"] == "2a4162859de0d19df809c1b31c6c2b8d2a31823e65d6ab36e6f2e7325545ebe8"
    assert d["lo"] == 255255 and d["hi"] == 40000000000254234 and d["survivors"] == 0
    assert d["primes"] == d["rung"] + d["direct"] + d["survivors"]
    assert d["table_sha256"].startswith("6af5e762")


def test_shard_0_rederived_on_gb300_matches_production():
    """Shard 0 of the reference's 250-shard run over [255255, 10^19) (data/c19/shard_0.meta, an
    L4 run), re-derived on one GB300 by the drop-in binary (its command and wall time are in the
    meta's header): the same certificate count, the same sha256 of the 394 M certificate lines in
    the same order, the same SUMMARY, the same filter table."""
    path = golden("metas", "gb300_shard_0.meta")
    if not os.path.exists(path):
        pytest.skip("no GB300 re-derivation of shard 0 committed")
    ref = shard_meta.parse_meta(read("metas", "c19_shard_0.meta"))
    got = shard_meta.parse_meta(open(path).read())
    assert got["complete"] and got["idx"] == 0 and got["nshards"] == 250 and got["rc"] == 0
    assert shard_meta.audit(ref, got) == []
    for k in ("certs", "cert_sha256", "lo", "hi", "positions", "covered", "mr", "composite", "rung", "direct",
              "survivors", "table_sha256"):
        assert got[k] == ref[k], k


def test_audit():
    a = shard_meta.parse_meta(read("metas", "c19_shard_0.meta"))
    assert shard_meta.audit(a, dict(a)) == []
    b = dict(a, certs=a["certs"] + 1, cert_sha256="0" * 64)
    assert shard_meta.audit(a, b) == ["certs 394469504 != 394469505", "cert_sha256 differs"]
    assert shard_meta.audit(a, b, compare_digest=False) == ["certs 394469504 != 394469505"]
    c = dict(a, complete=False)
    assert "incomplete meta (no SUMMARY)" in shard_meta.audit(a, c)


def test_round_order_is_a_permutation_by_round_then_lane():
    text = read("gen", "c2_gpu.out")
    lo = int(text.splitlines()[-1].split("lo=")[1].split()[0])
    body = "".join(ln for ln in text.splitlines(keepends=True) if not ln.startswith("SUMMARY"))
    import oracle
    classes = oracle.wheel(M)["classes"]
    r = shard_meta.round_order(body, lo, M, classes, 1024)
    assert sorted(r.splitlines()) == sorted(body.splitlines()) and r != body
    lane_of = {c: i for i, c in enumerate(classes)}
    keys = []
    for ln in r.splitlines():
        p = int(ln.split()[1])
        J = (p - (lo + (p % M - lo) % M)) // M
        keys.append((J // 1024, lane_of[p % M], J))
    assert keys == sorted(keys)
    assert shard_meta.round_order(body, lo, M, classes, 1 << 30) == body   # one round: lane order


def test_round_order_reproduces_the_production_w19_stream():
    """data/rederive/windows/w19_certificates.txt is the production driver's stream (two
    rounds of 262144 positions per lane): the oracle's lane-major text rearranged by
    round_order is that file byte for byte, and differs from the lane-major text."""
    import subprocess
    import oracle
    lo, hi = 5000000000000000000, 5000001000000000000
    out = subprocess.run([oracle.CLI, str(lo), str(hi), "--filters", GPU_TABLE], capture_output=True, text=True).stdout
    body = "".join(ln for ln in out.splitlines(keepends=True) if not ln.startswith("SUMMARY"))
    ref = read("windows", "w19_certificates.txt")
    rbody = "".join(ln for ln in ref.splitlines(keepends=True) if not ln.startswith("SUMMARY"))
    assert body != rbody
    assert shard_meta.round_order(body, lo, M, oracle.wheel(M)["classes"], 262144) == rbody


# ------------------------------------------------------------------ GPU
@pytest.mark.gpu
def test_cli_meta_reproduces_the_production_w19_digest(tmp_path):
    """The meta of the w19 window written on the GPU in the production order, in chunks of
    one round: cert_sha256 is the sha256 of the reference's own stream for that window."""
    lo, hi = 5000000000000000000, 5000001000000000000
    ref = read("windows", "w19_certificates.txt")
    certs, digest = shard_meta.stream_digest(ref)
    rc, meta = shard_meta.write_meta(str(tmp_path / "w19.meta"), lo, hi, filters=GPU_TABLE, order="round",
                                     chunk_rounds=1)
    assert rc == 0 and meta["complete"]
    assert meta["summary"] == ref.splitlines()[-1]
    assert meta["certs"] == certs == 8413
    assert meta["cert_sha256"] == digest


@pytest.mark.gpu
@pytest.mark.parametrize("order", ["round", "lane"])
def test_cli_meta_matches_digest_of_the_stream(order, tmp_path):
    import oracle
    lo, hi, seg = 10 ** 17 + 123456789, 10 ** 17 + 123456789 + (1 << 33), 512
    eng = es_sieve.Engine(wheel=M, filters=GPU_TABLE)
    try:
        text = eng.stream(lo, hi)
    finally:
        eng.close()
    body = "".join(ln for ln in text.splitlines(keepends=True) if not ln.startswith("SUMMARY"))
    if order == "round":
        body = shard_meta.round_order(body, lo, M, oracle.wheel(M)["classes"], seg)
    certs, digest = shard_meta.stream_digest(body)
    rc, meta = shard_meta.write_meta(str(tmp_path / "m.meta"), lo, hi, filters=GPU_TABLE, order=order, seg=seg,
                                     chunk_rounds=3)
    assert rc == 0 and meta["complete"]
    assert meta["summary"] == text.splitlines()[-1]
    assert meta["certs"] == certs and meta["cert_sha256"] == digest
    assert meta["order"] == order and meta["table_sha256"] == hashlib.sha256(open(GPU_TABLE, "rb").read()).hexdigest()
