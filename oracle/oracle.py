"""ctypes view of the CPU oracle (oracle/es_oracle.c -> oracle/_build/libes_oracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU
baseline leg, always as the checker of the GPU engine, never as part of it.
"""
import ctypes as C
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libes_oracle.so")
CLI = os.path.join(HERE, "_build", "es_oracle")
REF_DIR = os.path.join(HERE, "_ref")

_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        u64, P = C.c_uint64, C.POINTER
        L.es_o_is_prime.argtypes = [u64]; L.es_o_is_prime.restype = C.c_int
        L.es_o_sprp2.argtypes = [u64]; L.es_o_sprp2.restype = C.c_int
        L.es_o_is_prime_batch.argtypes = [C.c_void_p, C.c_size_t, C.c_void_p]; L.es_o_is_prime_batch.restype = None
        L.es_o_factor.argtypes = [u64, P(u64), P(C.c_int)]; L.es_o_factor.restype = C.c_int
        L.es_o_solve_rung.argtypes = [u64, C.c_char_p, C.c_size_t]; L.es_o_solve_rung.restype = C.c_int
        L.es_o_solve_direct.argtypes = [u64, C.c_char_p, C.c_size_t]; L.es_o_solve_direct.restype = C.c_int
        L.es_o_wheel.argtypes = [u64, P(u64), C.c_size_t, P(u64), P(u64), P(u64)]; L.es_o_wheel.restype = C.c_size_t
        L.es_o_default_filters.argtypes = [u64, u64, u64, P(u64), P(u64), C.c_size_t, P(C.c_size_t), P(u64)]
        L.es_o_default_filters.restype = C.c_size_t
        L.es_o_scan.argtypes = [u64, u64, u64, P(u64), P(u64), C.c_size_t, C.c_size_t, u64, C.c_int, C.c_int, P(u64)]
        L.es_o_scan.restype = C.c_void_p
        L.es_o_free.argtypes = [C.c_void_p]
        _lib = L
    return _lib


def is_prime(n):
    return bool(lib().es_o_sprp2(n) and lib().es_o_is_prime(n))


def is_prime_array(values):
    """Verdicts for a numpy uint64 array (threads over values): a uint8 array, 1 = prime."""
    import numpy as np
    v = np.ascontiguousarray(values, dtype=np.uint64)
    out = np.zeros(len(v), dtype=np.uint8)
    lib().es_o_is_prime_batch(v.ctypes.data, len(v), out.ctypes.data)
    return out


def factor(n):
    pr = (C.c_uint64 * 16)()
    ex = (C.c_int * 16)()
    k = lib().es_o_factor(n, pr, ex)
    return [(int(pr[i]), int(ex[i])) for i in range(k)]


def solve_rung(p):
    buf = C.create_string_buffer(200)
    return buf.value.decode() if lib().es_o_solve_rung(p, buf, 200) else None


def solve_direct(p):
    buf = C.create_string_buffer(200)
    return buf.value.decode() if lib().es_o_solve_direct(p, buf, 200) else None


def wheel(M):
    cls = (C.c_uint64 * 4096)()
    pm, fnv, f1 = C.c_uint64(), C.c_uint64(), C.c_uint64()
    n = lib().es_o_wheel(M, cls, 4096, C.byref(pm), C.byref(fnv), C.byref(f1))
    return {"classes": [int(cls[i]) for i in range(min(n, 4096))], "max_pmin": pm.value, "fnv64": fnv.value,
            "n_f1_only": f1.value}


def default_filters(M, mmax=10000, sieve_p=0):
    ncov, pmax = C.c_size_t(), C.c_uint64()
    n = lib().es_o_default_filters(M, mmax, sieve_p, None, None, 0, C.byref(ncov), C.byref(pmax))
    mods, ress = (C.c_uint64 * n)(), (C.c_uint64 * n)()
    lib().es_o_default_filters(M, mmax, sieve_p, mods, ress, n, C.byref(ncov), C.byref(pmax))
    return list(mods), list(ress), ncov.value


def scan(lo, hi, M, mods, ress, ncov, seg=262144, emit_survivors=True, threads=0):
    """(stream text without SUMMARY, counters dict) for [lo, hi), lanes merged in order."""
    n = len(mods)
    am, ar = (C.c_uint64 * max(n, 1))(*mods), (C.c_uint64 * max(n, 1))(*ress)
    cnt = (C.c_uint64 * 8)()
    p = lib().es_o_scan(lo, hi, M, am, ar, n, ncov, seg, 1 if emit_survivors else 0, threads, cnt)
    text = C.cast(p, C.c_char_p).value.decode()
    lib().es_o_free(p)
    names = ("positions", "covered", "sieved", "mr", "composite", "rung", "direct", "survivors")
    return text, {k: int(cnt[i]) for i, k in enumerate(names)}


def cli(args, timeout=600):
    """Run the oracle's rung_scan3-compatible CLI; returns (returncode, stdout, stderr)."""
    if not os.path.exists(CLI):
        build()
    r = subprocess.run([CLI] + [str(a) for a in args], capture_output=True, text=True, timeout=timeout)
    return r.returncode, r.stdout, r.stderr


def ref_binary(name):
    """Path of a reference scanner built from the reference sources, or None."""
    p = os.path.join(REF_DIR, name)
    return p if os.path.exists(p) else None
