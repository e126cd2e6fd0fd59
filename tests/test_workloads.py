"""The synthetic inputs match the configurations they stand in for: the 4096-window batch
(lengths floor(2^(16+12U)), heights log-uniform between the filter floor and the stage-E
ceiling), the serving arrivals (Poisson, mean gap 0.5 ms, lengths 2^12..2^30), the c3 window
(2^34 integers at height >= 1.7e19), all deterministic in the seed."""
import math
import statistics

import workloads


def test_batch_windows_shape_and_determinism():
    w = workloads.batch_windows(4096)
    assert w == workloads.batch_windows(4096) and w != workloads.batch_windows(4096, seed=workloads.SEED + 1)
    assert len(w) == 4096
    lens = [hi - lo for lo, hi in w]
    assert min(lens) >= 2 ** 16 and max(lens) < 2 ** 28
    assert all(lo > 255254 and hi <= workloads.DIRECT_PMAX for lo, hi in w)
    # log2(length) uniform on [16, 28): mean 22
    assert abs(statistics.mean(math.log2(x) for x in lens) - 22) < 0.3
    # heights log-uniform: half of them below the geometric midpoint of the range
    mid = math.sqrt(255255 * 1.8446744065e19)
    assert abs(sum(lo < mid for lo, _ in w) / len(w) - 0.5) < 0.05
    # about 1.3e11 integers a step (E[len] = (2^28 - 2^16) / (12 ln 2))
    assert 1.1e11 < sum(lens) < 1.6e11


def test_serve_requests_are_poisson_with_the_stated_gap():
    r = workloads.serve_requests(20000, seed=workloads.SEED + 1000)
    t = [x[0] for x in r]
    assert t == sorted(t)
    gaps = [b - a for a, b in zip(t, t[1:])]
    assert abs(statistics.mean(gaps) - 0.0005) < 0.00003
    lens = [hi - lo for _, lo, hi in r]
    assert min(lens) >= 2 ** 12 and max(lens) < 2 ** 30
    assert all(lo > 255254 and hi <= workloads.DIRECT_PMAX for _, lo, hi in r)


def test_c3_window():
    c = workloads.c3()
    assert c["hi"] - c["lo"] == 2 ** 34 and c["lo"] >= 17 * 10 ** 18 and c["hi"] <= workloads.DIRECT_PMAX
    assert c == workloads.c3()


def test_batch19_windows_shape():
    w = workloads.batch19_windows(4096)
    assert w == workloads.batch19_windows(4096) and len(w) == 4096
    lens = [hi - lo for lo, hi in w]
    assert min(lens) >= 2 ** 16 and max(lens) < 2 ** 28
    assert all(lo >= 10 ** 19 and hi <= workloads.DIRECT_PMAX for lo, hi in w)
    assert abs(statistics.mean(math.log2(x) for x in lens) - 22) < 0.3
    assert 1.1e11 < sum(lens) < 1.6e11


def test_committed_batch_windows_are_the_seeded_ones():
    """The fixtures keep the exact windows; on this host workloads.py draws the same ones."""
    import os
    gen = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "gen")
    assert workloads.read_windows(os.path.join(gen, "batch4096.windows")) == workloads.batch_windows(4096)
    assert workloads.read_windows(os.path.join(gen, "batch19_4096.windows")) == workloads.batch19_windows(4096)
