"""The C ABI without a GPU: the library loads, exports exactly what include/es_sieve.h
declares, formats records like the reference, and refuses to run without a device."""
import ctypes as C
import os
import re
import subprocess

import pytest

import es_sieve
from conftest import ROOT, golden, read

HEADER = os.path.join(ROOT, "include", "es_sieve.h")


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(es_sieve.LIB_PATH):
        import sys
        sys.path.insert(0, ROOT)
        import __graft_entry__
        __graft_entry__.build()
    return es_sieve.load_library()


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(es_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_boundary():
    names = declared_functions()
    for n in ("es_open", "es_close", "es_run_window", "es_run_batch", "es_submit", "es_poll", "es_free_records",
              "es_format_record", "es_format_summary", "es_is_prime_batch", "es_solve_rung_batch",
              "es_solve_direct_batch", "es_factor_batch"):
        assert n in names


def test_library_exports_every_declared_symbol(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", es_sieve.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(ln.split()[-1] for ln in out.splitlines() if ln.strip())
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing
    for n in declared_functions():
        getattr(lib, n)


def test_open_without_a_device_fails_loudly(lib):
    if os.path.exists("/dev/nvidia0") or os.path.exists("/dev/nvidiactl"):
        pytest.skip("a GPU is present")
    with pytest.raises(es_sieve.EsError) as ex:
        es_sieve.Engine(wheel=120120)
    assert ex.value.status == es_sieve.ES_ERR_CUDA


def _rec(**kw):
    r = {n: 0 for n in es_sieve.RECORD_DTYPE.names}
    r.update(kw)
    return r


def test_record_formats(lib):
    # RUNG with a 128-bit witness, SOLVED, SURVIVOR: the reference's line formats
    u = 2 ** 100 + 12345
    assert es_sieve.format_record(_rec(kind=1, p=5000000132492525161, a=1250000033123131291, b=3,
                                       c=u & (2 ** 64 - 1), d=u >> 64)) == \
        "RUNG 5000000132492525161 1250000033123131291 3 %d\n" % u
    assert es_sieve.format_record(_rec(kind=1, p=5, a=2, b=3, c=0, d=0)) == "RUNG 5 2 3 0\n"
    assert es_sieve.format_record(_rec(kind=2, p=9223372036854775837, a=1, b=2, c=3, d=4)) == \
        "SOLVED 9223372036854775837 1 2 3 4\n"
    assert es_sieve.format_record(_rec(kind=3, p=18446744065119614971)) == "SURVIVOR 18446744065119614971\n"
    assert es_sieve.format_record(_rec(kind=9)) == ""


def test_record_formats_random(lib):
    """Every width of every field, witnesses across the 2^64 and 10^19 boundaries."""
    import random
    rng = random.Random(5)
    us = [0, 1, 9, 10, 2 ** 64 - 1, 2 ** 64, 10 ** 19 - 1, 10 ** 19, 10 ** 19 + 1, 10 ** 38, 2 ** 126 - 1, 2 ** 127 - 1]
    us += [rng.getrandbits(rng.randint(1, 127)) for _ in range(2000)]
    for u in us:
        p, a, b = rng.getrandbits(64), rng.getrandbits(62), rng.randint(1, 255)
        assert es_sieve.format_record(_rec(kind=1, p=p, a=a, b=b, c=u & (2 ** 64 - 1), d=u >> 64)) == \
            "RUNG %d %d %d %d\n" % (p, a, b, u)
    for _ in range(500):
        v = [rng.getrandbits(rng.randint(1, 64)) for _ in range(5)]
        assert es_sieve.format_record(_rec(kind=2, p=v[0], a=v[1], b=v[2], c=v[3], d=v[4])) == \
            "SOLVED %d %d %d %d %d\n" % tuple(v)


def test_load_filters_errors(lib, tmp_path):
    m, r, n = C.POINTER(C.c_uint64)(), C.POINTER(C.c_uint64)(), C.c_size_t()
    assert lib.es_load_filters(b"/nonexistent/file", C.byref(m), C.byref(r), C.byref(n)) == es_sieve.ES_ERR_FILTERS
    empty = tmp_path / "empty.txt"
    empty.write_text("# no filters\n")
    assert lib.es_load_filters(str(empty).encode(), C.byref(m), C.byref(r), C.byref(n)) == es_sieve.ES_ERR_FILTERS
    path = golden("filters", "f_M2042040_mmax2000_gpu.txt").encode()
    assert lib.es_load_filters(path, C.byref(m), C.byref(r), C.byref(n)) == 0
    assert n.value == 3745 and m[0] == 19 and r[0] == 15
    lib.es_free_u64(m)
    lib.es_free_u64(r)


def test_status_strings(lib):
    for s in range(10):
        assert lib.es_status_str(s)


def test_cli_host_modes():
    cli = es_sieve.CLI_PATH
    if not os.path.exists(cli):
        pytest.skip("CLI not built")
    import hashlib
    want = dict(ln.split()[::-1] for ln in read("class_tables.sha256").splitlines())
    out = subprocess.run([cli, "--dump-classes", "--wheel", "120120"], capture_output=True).stdout
    assert hashlib.sha256(out).hexdigest() == want["class_table_120120.txt"]
    r = subprocess.run([cli, "1000000000000", "1000200000000", "--bogus"], capture_output=True, text=True)
    assert r.returncode == 1 and "unknown option" in r.stderr
    r = subprocess.run([cli], capture_output=True, text=True)
    assert r.returncode == 1 and "usage" in r.stderr


def test_cli_dump_classes_2042040():
    cli = es_sieve.CLI_PATH
    if not os.path.exists(cli):
        pytest.skip("CLI not built")
    import hashlib
    want = dict(ln.split()[::-1] for ln in read("class_tables.sha256").splitlines())
    out = subprocess.run([cli, "--dump-classes"], capture_output=True).stdout
    assert hashlib.sha256(out).hexdigest() == want["class_table_2042040.txt"]


# (ctypes mirror in es_sieve.py, the C struct it stands for); field names match
_LAYOUTS = [
    (es_sieve.Config, "es_config"),
    (es_sieve.Counters, "es_counters"),
    (es_sieve.Record, "es_record"),
    (es_sieve.Records, "es_records"),
    (es_sieve.Window, "es_window"),
    (es_sieve.Info, "es_info_t"),
    (es_sieve.Schedule, "es_schedule"),
    (es_sieve.Timing, "es_timing_t"),
]


def test_struct_layouts_match_the_header(tmp_path):
    """Every ctypes structure the Python binding passes across the boundary has the size and
    field offsets of its C declaration (a C program compiled against include/es_sieve.h
    prints them)."""
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "es_sieve.h"', "int main(void) {"]
    for cls, cname in _LAYOUTS:
        lines.append('  printf("%s size %%zu\\n", sizeof(%s));' % (cname, cname))
        for fname, _t in cls._fields_:
            lines.append('  printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (cname, fname, cname, fname))
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = str(tmp_path / "layout")
    subprocess.run(["gcc", "-std=c11", "-I", os.path.dirname(HEADER), str(src), "-o", exe], check=True)
    out = dict(line.rsplit(" ", 1) for line in subprocess.run([exe], capture_output=True, text=True,
                                                              check=True).stdout.splitlines())
    for cls, cname in _LAYOUTS:
        assert int(out["%s size" % cname]) == C.sizeof(cls), cname
        for fname, _t in cls._fields_:
            assert int(out["%s.%s" % (cname, fname)]) == getattr(cls, fname).offset, (cname, fname)


def test_cli_self_test_wheel_checks_pass_on_the_host():
    """--verify's host checks (the class-table derivation against the constants of
    sieve/rung_scan3.cpp:821-897) pass without a GPU; only the device line needs one."""
    cli = es_sieve.CLI_PATH
    if not os.path.exists(cli):
        pytest.skip("CLI not built")
    out = subprocess.run([cli, "--verify"], capture_output=True, text=True).stdout
    host = [ln for ln in out.splitlines() if ln.startswith("  ") and "device" not in ln]
    assert len(host) == 14
    assert all(ln.startswith("  pass ") for ln in host), out
