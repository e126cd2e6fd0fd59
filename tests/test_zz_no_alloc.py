"""The allocation-free primality entry point (es_is_prime_noalloc).

It is for callers that cannot allocate device memory themselves -- a process whose device
memory is reserved up front by someone else, code where an allocation may not block or fail
at run time, a framework that owns every device allocation -- and hands them a primality
test over buffers they already hold on the device, with its scratch in a fixed array of the
library's device image instead of memory from cudaMalloc.

This file runs last (pytest collects it after the others), so a run that stops at the
first failure has already run every other test. The test is the caller here: it allocates
the input and output buffers with torch; the entry point itself allocates nothing.
"""
import ctypes as C

import numpy as np
import pytest

import es_sieve
import oracle
import workloads

pytestmark = pytest.mark.gpu

NOALLOC_MAX = 1 << 20   # ES_NOALLOC_MAX in include/es_sieve.h


def _values(seed, count):
    """Dense odd runs at several heights (primes and composites), random u64, small values."""
    g = workloads.SplitMix64(seed)
    parts = [np.arange(0, 200, dtype=np.uint64)]
    for base in (10 ** 9, 2 ** 62 + 1, 2 ** 63 - 999, 18446744065119000001, 2 ** 64 - 4001):
        parts.append(np.arange(base, base + 2000, 2, dtype=np.uint64))
    parts.append(np.array([g.next() for _ in range(count)], dtype=np.uint64))
    return np.concatenate(parts)[:count]


def _run(lib, torch, vals, stream=None):
    """One call on `stream` (a torch.cuda.Stream; None: the current stream), its output read
    back after that stream has finished."""
    d_n = torch.from_numpy(vals.view(np.int64).copy()).cuda()
    d_out = torch.full((len(vals),), 7, dtype=torch.uint8, device="cuda")   # 7: never a verdict
    torch.cuda.synchronize()
    s = stream if stream is not None else torch.cuda.current_stream()
    st = lib.es_is_prime_noalloc(C.c_void_p(d_n.data_ptr()), len(vals), C.c_void_p(d_out.data_ptr()),
                                 C.c_void_p(s.cuda_stream))
    assert st == es_sieve.ES_OK
    s.synchronize()
    return d_out.cpu().numpy()


def _check(got, vals, eng):
    """Against the CPU oracle's Miller-Rabin (an independent restatement of the reference's
    sprp2 && is_prime) and against the allocating entry point of the same library."""
    assert set(np.unique(got).tolist()) <= {0, 1}
    assert np.array_equal(got, oracle.is_prime_array(vals))
    assert np.array_equal(got.astype(bool), eng.is_prime(vals))
    assert 0 < got.sum() < len(vals)


def test_no_alloc_matches_the_oracle_and_the_allocating_entry_point_on_two_calls():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    lib = es_sieve.load_library()
    with es_sieve.Engine(wheel=120120) as eng:
        # two calls in a row; the second is shorter, so entries the first call left in the
        # shared scratch array would show up as wrong verdicts if the reset were missing
        for seed, count in ((11, 60000), (12, 5003)):
            vals = _values(seed, count)
            _check(_run(lib, torch, vals), vals, eng)


def test_no_alloc_at_its_maximum_on_a_side_stream():
    """count == ES_NOALLOC_MAX fills the scratch list to its last slot when every value
    passes the base-2 round (here: a list of primes and base-2 strong pseudoprimes, repeated);
    then a mixed call on a non-default stream, read after that stream alone is synchronised."""
    torch = pytest.importorskip("torch")
    lib = es_sieve.load_library()
    with es_sieve.Engine(wheel=120120) as eng:
        base = _values(21, 40000)
        passers = base[oracle.is_prime_array(base).astype(bool)]
        psp2 = np.array([2047, 3277, 4033, 4681, 8321, 3215031751, 1122004669633], dtype=np.uint64)
        pool = np.concatenate([passers, psp2])
        vals = np.resize(pool, NOALLOC_MAX)
        _check(_run(lib, torch, vals), vals, eng)
        side = torch.cuda.Stream()
        vals = _values(22, 30011)
        _check(_run(lib, torch, vals, side), vals, eng)


def test_no_alloc_refuses_more_than_its_maximum():
    torch = pytest.importorskip("torch")
    lib = es_sieve.load_library()
    d_n = torch.zeros(4, dtype=torch.int64, device="cuda")
    d_out = torch.zeros(4, dtype=torch.uint8, device="cuda")
    # refused before any device work: the buffers are never touched
    st = lib.es_is_prime_noalloc(C.c_void_p(d_n.data_ptr()), NOALLOC_MAX + 1, C.c_void_p(d_out.data_ptr()), None)
    assert st == es_sieve.ES_ERR_ARG
    assert lib.es_is_prime_noalloc(None, 0, None, None) == es_sieve.ES_OK
