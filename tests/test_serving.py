"""Serving: continuously batched requests give the reference's results.

Requests arrive while others are on the GPU (a submitting thread paced like Poisson
arrivals, lengths log-uniform up to 2^30 as in the serving configuration) and are batched with
whatever else is queued when a serving stream frees up. Every request's counters and records
must equal those of the same windows run alone; requests whose windows the reference itself
scanned (the 48 golden batch windows) must give its stream byte for byte, and a few small
requests must give the CPU oracle's."""
import threading
import time

import pytest

import es_sieve
import oracle
import workloads
from conftest import golden, read, split_stream

pytestmark = pytest.mark.gpu

GPU_TABLE = golden("filters", "f_M2042040_mmax2000_gpu.txt")


@pytest.fixture(scope="module")
def eng():
    e = es_sieve.Engine(wheel=2042040, filters=GPU_TABLE)
    yield e
    e.close()


def _requests(n, seed):
    reqs = workloads.serve_requests(n, seed=seed, lmax_log2=30)
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


def _serve_all(eng, reqs, gap_s=0.0003):
    """Submit [windows] requests paced gap_s apart from a thread; poll them in order."""
    tickets = [None] * len(reqs)

    def submitter():
        for i, wins in enumerate(reqs):
            time.sleep(gap_s)
            tickets[i] = eng.submit(wins)

    th = threading.Thread(target=submitter)
    th.start()
    out = []
    for i in range(len(reqs)):
        while tickets[i] is None:
            time.sleep(0.0002)
        out.append(eng.poll(tickets[i], len(reqs[i]), timeout_ms=60000))
    th.join()
    return out


def test_served_requests_match_the_reference_and_the_oracle(eng):
    """The 48 golden batch windows (reference records from its own sweep_lane), one request
    each, interleaved with serving traffic; then small requests against the CPU oracle."""
    wins = workloads.read_windows(golden("gen", "batch48.windows"))
    want = read("gen", "batch48.out").splitlines(keepends=True)
    per_window, cur = [], []
    for ln in want:                       # the reference stream, cut at each SUMMARY
        cur.append(ln)
        if ln.startswith("SUMMARY "):
            per_window.append("".join(cur))
            cur = []
    traffic = [[(lo, hi)] for _, lo, hi in workloads.serve_requests(48, seed=5)]
    reqs = [r for pair in zip([[w] for w in wins], traffic) for r in pair]
    res = _serve_all(eng, reqs)
    for k, (lo, hi) in enumerate(wins):
        per, recs = res[2 * k]
        assert eng.text(lo, hi, per[0], recs) == per_window[k]
    mods, ress = es_sieve.load_filters(GPU_TABLE)
    mods, ress = [int(m) for m in mods], [int(r) for r in ress]
    small = [(lo, lo + (1 << 20)) for _, lo, _ in workloads.serve_requests(4, seed=77)]
    res = _serve_all(eng, [[w] for w in small])
    for (lo, hi), (per, recs) in zip(small, res):
        text, cnt = oracle.scan(lo, hi, 2042040, mods, ress, len(mods))
        got = eng.text(lo, hi, per[0], recs)
        assert split_stream(got)[0] == split_stream(text)[0]
        assert per[0] == cnt


def test_one_poller_per_ticket(eng):
    """A second es_poll on a ticket another thread is waiting on is refused (ES_ERR_ARG) instead
    of reading a request the first poller is about to free; the first poller gets the result."""
    wins = [(10 ** 19 + k * (1 << 41), 10 ** 19 + k * (1 << 41) + (1 << 40)) for k in range(24)]
    t = eng.submit(wins)
    got = {}

    def first():
        while "r" not in got:
            try:
                got["r"] = eng.poll(t, len(wins), timeout_ms=-1)
            except es_sieve.EsError as ex:  # the main thread's check held the claim for a moment
                if "already being polled" not in str(ex):
                    raise
                time.sleep(0.0005)

    th = threading.Thread(target=first)
    th.start()
    refused = False
    while th.is_alive() and not refused:
        try:
            eng.poll(t, len(wins), timeout_ms=0)
            break                         # the first poller had not claimed it yet and it finished
        except es_sieve.EsError as ex:
            if ex.status == es_sieve.ES_ERR_ARG and "already being polled" in str(ex):
                refused = True
            elif ex.status != es_sieve.ES_ERR_TIMEOUT:
                break                     # unknown ticket: the first poller already took it
        time.sleep(0.001)
    th.join()
    assert refused
    per, recs = got["r"]
    alone_c, alone_r = eng.run_batch(wins)
    assert per == alone_c and recs.tobytes() == alone_r.tobytes()


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
