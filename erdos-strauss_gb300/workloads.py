"""Seeded synthetic workloads for the verification sieve (all integer, all reproducible).

PRNG: splitmix64, default seed 0xE52026. The reference measures on no public suite; these
stand in for its configurations with the same shapes, sizes and distributions:

  c1     2^26 consecutive integers from 10^9, wheel 120120, the 120120 runtime filter table
  c2     2^34 integers from a seeded offset in [10^15, 2*10^15), wheel 2042040, gpu table
  c3     2^34 integers from a seeded offset in [1.7e19, DIRECT_PMAX - 2^34], same table
  batch  4096 windows, lengths floor(2^(16 + 12 U1)), starts
         floor(exp(ln 255255 + U2 (ln 1.8446744065e19 - ln 255255))), clamped into
         [255255, DIRECT_PMAX - len]
  batch19  the same length law, starts log-uniform over [10^19, DIRECT_PMAX - len]: the
         batched configuration at the height the run19/run64 shards cover
  serve  Poisson arrivals (mean gap 0.5 ms), lengths log-uniform in [2^12, 2^30], starts as
         for the batch
"""
import math

MASK = (1 << 64) - 1
SEED = 0xE52026
DIRECT_PMAX = 18446744065119614976        # (2^32-1)^2 - 2048 - 1
FLOOR_2042040 = 255254                    # wheel_pmin of the 2042040 table
TOP = 18446744065000000000                # 1.8446744065e19, the batch's upper height
BASE19 = 10 ** 19                         # lowest start of the batch at the top of the range


class SplitMix64:
    def __init__(self, seed=SEED):
        self.state = seed & MASK

    def next(self):
        self.state = (self.state + 0x9E3779B97F4A7C15) & MASK
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK
        return z ^ (z >> 31)

    def uniform(self):
        """U in [0, 1) with 53 random bits."""
        return (self.next() >> 11) * (1.0 / (1 << 53))


def c1():
    return {"name": "c1", "lo": 10 ** 9, "hi": 10 ** 9 + (1 << 26), "wheel": 120120,
            "filters": "f_M120120_mmax2000_runtime.txt"}


def c2(seed=SEED):
    g = SplitMix64(seed)
    lo = 10 ** 15 + g.next() % 10 ** 15
    return {"name": "c2", "lo": lo, "hi": lo + (1 << 34), "wheel": 2042040,
            "filters": "f_M2042040_mmax2000_gpu.txt"}


def c3(seed=SEED):
    g = SplitMix64(seed)
    base = 17 * 10 ** 18
    span = DIRECT_PMAX - (1 << 34) - base + 1
    lo = base + g.next() % span
    return {"name": "c3", "lo": lo, "hi": lo + (1 << 34), "wheel": 2042040,
            "filters": "f_M2042040_mmax2000_gpu.txt"}


def _height(g, lo_min, top):
    return int(math.exp(math.log(lo_min) + g.uniform() * (math.log(top) - math.log(lo_min))))


def batch_windows(n=4096, seed=SEED, lmin_log2=16, lmax_log2=28, lo_min=FLOOR_2042040 + 1):
    """The batched configuration: n windows of uneven length and height."""
    g = SplitMix64(seed)
    out = []
    for _ in range(n):
        length = int(2.0 ** (lmin_log2 + (lmax_log2 - lmin_log2) * g.uniform()))
        lo = _height(g, lo_min, TOP)
        lo = max(lo, lo_min)
        lo = min(lo, DIRECT_PMAX - length)
        out.append((lo, lo + length))
    return out


def batch19_windows(n=4096, seed=SEED, lmin_log2=16, lmax_log2=28):
    """The batched configuration at the top of the range: the same length law as
    batch_windows, starts log-uniform over [10^19, DIRECT_PMAX - len]."""
    g = SplitMix64(seed ^ 0x19)
    out = []
    for _ in range(n):
        length = int(2.0 ** (lmin_log2 + (lmax_log2 - lmin_log2) * g.uniform()))
        top = DIRECT_PMAX - length
        lo = min(max(_height(g, BASE19, top), BASE19), top)
        out.append((lo, lo + length))
    return out


def read_windows(path):
    """Windows from a file of "LO HI" lines (the committed fixtures keep the exact windows,
    so that a platform whose libm rounds exp or log differently still runs the same ones)."""
    out = []
    with open(path) as f:
        for ln in f:
            t = ln.split()
            if len(t) == 2:
                out.append((int(t[0]), int(t[1])))
    return out


def serve_requests(n, seed=SEED, mean_gap_s=0.0005, lmin_log2=12, lmax_log2=30, lo_min=FLOOR_2042040 + 1):
    """Serving arrivals: (arrival_time_s, lo, hi), Poisson with the given mean gap."""
    g = SplitMix64(seed ^ 0x5E12E)
    t = 0.0
    out = []
    for _ in range(n):
        t += -math.log(1.0 - g.uniform()) * mean_gap_s
        length = int(2.0 ** (lmin_log2 + (lmax_log2 - lmin_log2) * g.uniform()))
        lo = min(max(_height(g, lo_min, TOP), lo_min), DIRECT_PMAX - length)
        out.append((t, lo, lo + length))
    return out


def shard_bounds(lo, hi, i, n):
    """Ceil-span tiling of [lo, hi) into n shards (sieve/rung_scan3.cpp:1022-1027)."""
    if n <= 1:
        return lo, hi
    span = (hi - lo + n - 1) // n
    a = lo + i * span
    b = min(hi, a + span)
    return a, max(a, b)
