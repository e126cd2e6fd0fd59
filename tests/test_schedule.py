"""Schedules and the autotuner: every schedule gives the same counters and records.

The run-time schedule moves windows between the short-window kernel and the segment
marking (short_max) and resizes the stage-D grid; neither may change a result. The checks run
the batched sample and windows either side of each short_max boundary under every candidate
schedule and compare with the default, byte for byte."""
import pytest

import es_sieve
import workloads
from conftest import golden, read

pytestmark = pytest.mark.gpu

GPU_TABLE = golden("filters", "f_M2042040_mmax2000_gpu.txt")
M = 2042040


@pytest.fixture(scope="module")
def eng():
    e = es_sieve.Engine(wheel=M, filters=GPU_TABLE)
    yield e
    e.close()


def _smax(eng):
    """The engine's largest short_max: its default schedule's (the kill-mask repeat)."""
    return eng.info()["short_max_limit"]


def _windows():
    wins = [tuple(int(x) for x in ln.split()) for ln in read("gen", "batch48.windows").splitlines()]
    g = workloads.SplitMix64(4242)
    for per_lane in (1, 31, 32, 33, 63, 64, 65, 127, 128, 129, 255, 256, 257, 300):
        lo = 10 ** 15 + g.next() % 10 ** 18
        wins.append((lo, lo + per_lane * M - g.next() % 1000))
    return wins


def test_every_schedule_gives_identical_results(eng):
    wins = _windows()
    top = _smax(eng)
    eng.set_schedule(short_max=top, rung_blocks_per_sm=6, long_split=0)
    base_c, base_r = eng.run_batch(wins)
    for split in (0, 1):
        for sm in sorted({1, 32, top // 2, top - 1, top}):
            for rb in (1, 4, 8, 16):
                eng.set_schedule(short_max=sm, rung_blocks_per_sm=rb, long_split=split)
                for sched in (es_sieve.ES_SCHED_PERSISTENT, es_sieve.ES_SCHED_PLAIN):
                    c, r = eng.run_batch(wins, schedule=sched)
                    assert c == base_c, (split, sm, rb, sched)
                    assert r.tobytes() == base_r.tobytes(), (split, sm, rb, sched)
    eng.set_schedule(short_max=top, rung_blocks_per_sm=6, long_split=1)


def test_long_windows_split_or_segmented_agree(eng):
    """Windows of 2^34 to 2^40 integers (8 K to 540 K positions per lane, so thousands of
    sub-windows) under both long-window schedules, against each other and against the
    golden c3 stream."""
    wins = [(workloads.c3()["lo"], workloads.c3()["hi"]), (10 ** 16 + 7, 10 ** 16 + 7 + (1 << 40)),
            (255255 + 1, 255255 + 1 + (1 << 38))]
    out = {}
    for split in (1, 0):
        eng.set_schedule(long_split=split)
        out[split] = eng.run_batch(wins)
    eng.set_schedule(long_split=1)
    assert out[0][0] == out[1][0]
    assert out[0][1].tobytes() == out[1][1].tobytes()
    c, r = out[1]
    mine = r[r["window"] == 0]
    assert eng.text(wins[0][0], wins[0][1], c[0], mine) == read("gen", "c3_gpu.out")


def test_autotune_picks_a_candidate_and_keeps_results(eng):
    wins = workloads.batch_windows(256, seed=77)
    before_c, before_r = eng.run_batch(wins)
    chosen = eng.autotune(wins, repeats=1)
    top = _smax(eng)
    assert chosen["short_max"] in (top // 4, top // 2, top) and chosen["rung_blocks_per_sm"] in (4, 6, 8)
    assert chosen["long_split"] in (0, 1)
    assert eng.schedule() == chosen
    c, r = eng.run_batch(wins)
    assert c == before_c and r.tobytes() == before_r.tobytes()
    eng.set_schedule(short_max=top, rung_blocks_per_sm=6, long_split=1)


def test_schedule_refusals(eng):
    top = _smax(eng)
    for kw in (dict(short_max=0), dict(short_max=top + 1), dict(rung_blocks_per_sm=0), dict(rung_blocks_per_sm=17)):
        with pytest.raises(es_sieve.EsError) as ex:
            eng.set_schedule(**kw)
        assert ex.value.status == es_sieve.ES_ERR_ARG
    assert eng.schedule() == {"short_max": top, "rung_blocks_per_sm": 6, "long_split": 1}
    with pytest.raises(es_sieve.EsError) as ex:
        eng.set_schedule(long_split=2)
    assert ex.value.status == es_sieve.ES_ERR_ARG
    with pytest.raises(es_sieve.EsError) as ex:
        eng.autotune([], repeats=1)
    assert ex.value.status == es_sieve.ES_ERR_ARG
