"""Serving: continuously batched requests give the same results as each request run alone.

Requests arrive while others are on the GPU (a submitting thread paced like Poisson
arrivals) and are batched with whatever else is queued when a serving stream frees up; every
request's counters and records must equal those of the same windows run alone."""
import threading
import time

import pytest

import es_sieve
import workloads
from conftest import golden

pytestmark = pytest.mark.gpu

GPU_TABLE = golden("filters", "f_M2042040_mmax2000_gpu.txt")


@pytest.fixture(scope="module")
def eng():
    e = es_sieve.Engine(wheel=2042040, filters=GPU_TABLE)
    yield e
    e.close()


def _requests(n, seed):
    reqs = workloads.serve_requests(n, seed=seed, lmax_log2=27)   # keep the test short
    out = []
    for i, (t, lo, hi) in enumerate(reqs):
        if i % 7 == 3:                              # some requests carry several windows
            out.append((t, [(lo, hi), (hi, hi + 12345), (lo // 2 + 300000, lo // 2 + 300000 + 99999)]))
        else:
            out.append((t, [(lo, hi)]))
    return out


def test_each_result_is_the_same_alone_and_in_the_mix(eng):
    reqs = _requests(160, seed=99)
    tickets = [None] * len(reqs)
    t0 = time.perf_counter()

    def submitter():
        for i, (t, wins) in enumerate(reqs):
            delay = t0 + t - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            tickets[i] = eng.submit(wins)

    th = threading.Thread(target=submitter)
    th.start()
    results = []
    for i in range(len(reqs)):
        while tickets[i] is None:
            time.sleep(0.0002)
        results.append(eng.poll(tickets[i], len(reqs[i][1]), timeout_ms=60000))
    th.join()
    for (t, wins), (per, recs) in zip(reqs, results):
        alone_c, alone_r = eng.run_batch(wins)
        assert per == alone_c
        assert recs.tobytes() == alone_r.tobytes()


def test_admission_and_refusals():
    small = es_sieve.Engine(wheel=2042040, filters=GPU_TABLE, mem_budget=1 << 20)
    try:
        with pytest.raises(es_sieve.EsError) as ex:
            small.submit([(10 ** 15, 10 ** 15 + (1 << 34))])       # needs far more than 1 MB
        assert ex.value.status == es_sieve.ES_ERR_BUSY
        with pytest.raises(es_sieve.EsError) as ex:
            small.submit([(100, 10 ** 9)])                          # below the pmin floor
        assert ex.value.status == es_sieve.ES_ERR_RANGE
        t = small.submit([(10 ** 12, 10 ** 12 + 10 ** 6)])         # small enough to admit
        per, recs = small.poll(t, 1, timeout_ms=60000)
        alone, _ = small.run_window(10 ** 12, 10 ** 12 + 10 ** 6)
        assert per[0] == alone
        with pytest.raises(es_sieve.EsError) as ex:
            small.poll(t, 1, timeout_ms=0)                          # the ticket is gone
        assert ex.value.status == es_sieve.ES_ERR_ARG
    finally:
        small.close()
