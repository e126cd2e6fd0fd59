#!/usr/bin/env python3
"""A filter table tuned for this engine's cost model (GB300), from the certified candidates.

The reference prunes its filter table for a per-mark cost: each filter is a progression the
scanner walks bit by bit, plus (on its CUDA port) a per-(lane, filter) offset setup, so a
filter pays for every mark (sieve/prune_filters.py, its cost constants and greedy). This engine
marks short windows from kill masks instead (one precomputed row per lane and distinct
stride s = mod / gcd(M, mod), holding every filter of that stride; rounds of 32 strides,
densest first, until every position of the segment is dead). That changes what a filter
costs:

  * a filter whose stride is already masked costs nothing per batch: it only makes the
    stride's mask denser (the row is built once, at es_open);
  * a stride costs one mask extraction per 32-position chunk of every segment that is still
    alive when its round comes: cheap for a stride that kills a lot early, dear for one that
    only matters to the segments with a survivor (those run every round);
  * a survivor costs a Miller-Rabin round (k_mr), and a prime survivor a rung walk (k_rung)
    and an emitted certificate;
  * the masks of all masked strides must fit the per-lane shared-memory budget (48 KB); a
    stride past it is walked filter by filter from the first-hit table (much dearer).

So the tuner chooses STRIDES, not filters: every certified candidate of a chosen stride is
kept. Candidates are the reference's two certified families (both derived here, in code of
this module): F1 covers m = 4acd - 1 <= mmax with m not dividing M, killing p = -4a^2 d
(mod m); F2 uniform rung certificates (r <= 63, u <= 64, gcd(r, u) = 1, L = 4ru not dividing
M), killing the residues rho (mod L) at which u | (pA)^2 and pA = -u (mod r), A = (p + r)/4.
Any subset of them is sound (dropping or adding a certified filter changes only which
primes reach stage D), so a tuned table is a speed choice and never a correctness one; it is
shipped beside the reference's table with its own digest and is never the parity default.

Model. Strides are ordered by kill density (sum over their filters of lanes hit / s, the
order k_mark_short walks them). On evaluation domains -- every lane, NPOS consecutive
positions from each of several anchors spread over the range in log scale -- each position
gets the rank of the first stride that kills it. A table made of the first k strides of that order then has, exactly and for every k at
once: survivors = positions whose rank is >= k; rounds of a task (two lanes x a segment of
z positions) = ceil((max rank + 1) / 32), or every round of the table when the task keeps a
survivor. The batch's tasks have the segment sizes of its windows (positions per lane, cut
at short_max), so the per-task figures are weighted by that histogram. Primes among the
survivors are counted with a deterministic Miller-Rabin (the 12 bases of the scanners).

    k_mark_short = a0 + a1 * rounds      k_mr = b0 + b1 * survivors
    k_rung       = c0 + c1 * primes      device time per batch = their sum

(the intercepts hold what does not move with the table: the tasks' set-up, the latency of
stage D's hardest factorization). The constants are measured on the GPU (`--calibrate FILE`:
es_timing's per-kernel times of the 4096-window batch under a sweep of prefix tables) and
fitted by least squares, one line per kernel; the tuned table is the prefix k with the least
modelled time among those whose masks fit the budget.

Usage:
  python filter_tune.py --report                                       the model per prefix
  python filter_tune.py --prefixes 64,96,128 --out DIR                 candidate tables
  python filter_tune.py --measure FILE --prefixes 64,96,...            time them on the GPU
  python filter_tune.py --calibrate FILE --write TABLE                 fit, write the tuned table

The shipped table (tables/f_M2042040_mmax2000_gb300.txt) was made by the last command from
tables/calibration_batch4096.json, which --measure wrote on one GB300.
"""
import argparse
import hashlib
import json
import math
import os
import sys
from math import gcd

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

M_DEFAULT = 2042040
SEG_SMALL = 128                 # kill-mask repeat of this build (positions past s)
MASK_WORDS_MAX = 48 * 1024 // 4  # per-lane mask budget, 32-bit words
SMD_MAX = 512                   # masked strides the short-window kernel stages
# Evaluation domains: every lane, NPOS positions from each anchor. The anchors are spread
# over the verified range in log scale, as the batched configuration's heights are: survivor
# density is not the same everywhere (below ~1e10 perfect squares, which no cover kills, are
# most of the survivors; above it the covers decide).
ANCHORS = tuple(10 ** e for e in (6, 8, 10, 12, 14, 16, 18))
NPOS = 1024
MR_BASES = (2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37)


# ------------------------------------------------------------------ certified candidates

def f1_covers(mmax, M):
    """(m, res) of every F1 cover with m <= mmax and m not dividing M: for each modulus
    m = 3 (mod 4), the ordered factorizations a*c*d of (m + 1) / 4."""
    out = set()
    for m in range(3, mmax + 1, 4):
        if M % m == 0:
            continue
        t = (m + 1) // 4
        for a in range(1, t + 1):
            if t % a:
                continue
            rest = t // a
            for c in range(1, rest + 1):
                if rest % c:
                    continue
                d = rest // c
                out.add((m, (-4 * a * a * d) % m))
    return sorted(out)


def f2_certs(M, rmax=63, umax=64):
    """(L, rho) of every uniform rung certificate with L = 4ru not dividing M. For
    p = rho (mod L), rho = -r (mod 4), q = p (p + r) / 4 is fixed mod ru, so one evaluation at
    p = rho decides both conditions (u | q^2, q = -u (mod r)) for the whole class."""
    out = set()
    for r in range(1, rmax + 1):
        for u in range(1, umax + 1):
            if gcd(r, u) != 1:
                continue
            L = 4 * r * u
            if M % L == 0:
                continue
            for rho in range((-r) % 4, L, 4):
                q = rho * ((rho + r) // 4)
                if (q % u) * (q % u) % u == 0 and (q + u) % r == 0:
                    out.add((L, rho))
    return sorted(out)


def candidates(mmax, M):
    """[(mod, res, family)] of both families, F1 first."""
    return [(m, r, "F1") for m, r in f1_covers(mmax, M)] + [(L, r, "F2") for L, r in f2_certs(M)]


# ------------------------------------------------------------------ the wheel's lanes

def wheel_lanes(M):
    """The unit classes mod M that no certificate with modulus dividing M kills (the wheel's
    lanes, ascending): F1 covers m | M, then F2 certificates L | M."""
    x = np.arange(M, dtype=np.int64)
    live = np.gcd(x, M) == 1
    for m in range(3, M + 1, 4):
        if M % m:
            continue
        t = (m + 1) // 4
        for a in range(1, t + 1):
            if t % a:
                continue
            rest = t // a
            for c in range(1, rest + 1):
                if rest % c == 0:
                    live[(-4 * a * a * (rest // c)) % m::m] = False
    for r in range(1, 64):
        for u in range(1, 65):
            L = 4 * r * u
            if gcd(r, u) != 1 or M % L:
                continue
            for rho in range((-r) % 4, L, 4):
                q = rho * ((rho + r) // 4)
                if (q % u) * (q % u) % u == 0 and (q + u) % r == 0:
                    live[rho::L] = False
    return np.nonzero(live)[0].astype(np.int64)


# ------------------------------------------------------------------ strides and hits

def stride_groups(cands, M, lanes):
    """{s: [(mod, res, family, lanes_hit_mask, K0 per hit lane)]} and each stride's kill
    density (sum over its filters of lanes hit / s), as k_mark_short orders them."""
    groups = {}
    for mod, res, fam in cands:
        g = gcd(M, mod)
        s = mod // g
        hit = ((res - lanes) % g) == 0
        if not hit.any():
            continue
        inv = pow((M // g) % s, -1, s) if s > 1 else 0
        k0 = (((res - lanes[hit]) // g) % s) * inv % s if s > 1 else np.zeros(int(hit.sum()), dtype=np.int64)
        groups.setdefault(s, []).append((mod, res, fam, hit, k0))
    dens = {s: sum(int(f[3].sum()) / s for f in fs) for s, fs in groups.items()}
    return groups, dens


def mask_words(s):
    return (s + SEG_SMALL + 31) // 32 + 1


def first_kill_ranks(order, groups, M, lanes, lo_ref, npos=NPOS):
    """rank[lane, j]: index in `order` of the first stride killing position j of the lane in
    the domain (positions K0_lane + j, K0_lane the lane's first position >= lo_ref); len(order)
    when none does."""
    L = len(lanes)
    kbase = (lo_ref - lanes + M - 1) // M                 # first K with rho + M K >= lo_ref
    rank = np.full((L, npos), len(order), dtype=np.int32)
    for i, s in enumerate(order):
        for mod, res, fam, hit, k0 in groups[s]:
            li = np.nonzero(hit)[0]
            j0 = (k0 - kbase[li]) % s                     # first hit index in the domain
            reps = (npos + s - 1) // s
            js = j0[:, None] + s * np.arange(reps)[None, :]
            ok = js < npos
            rows = np.broadcast_to(li[:, None], js.shape)[ok]
            cols = js[ok]
            cur = rank[rows, cols]
            rank[rows, cols] = np.minimum(cur, i)
    return rank, kbase


def is_prime(n):
    if n < 2:
        return False
    for p in MR_BASES:
        if n % p == 0:
            return n == p
    d, r = n - 1, 0
    while d % 2 == 0:
        d //= 2
        r += 1
    for a in MR_BASES:
        x = pow(a, d, n)
        if x in (1, n - 1):
            continue
        for _ in range(r - 1):
            x = x * x % n
            if x == n - 1:
                break
        else:
            return False
    return True


# ------------------------------------------------------------------ the model

def segment_histogram(windows, M, nlanes, short_max=64):
    """{z: tasks} of a batch under the split schedule: each window's lanes hold about
    len / M positions; windows longer than short_max per lane are cut into sub-windows of
    short_max positions; a task is a lane pair of one (sub-)window with a position."""
    hist = {}
    for lo, hi in windows:
        per = (hi - lo) / M
        if per < 1:                                       # fewer positions than lanes
            tasks, z = max(1.0, per * nlanes / 2), 1
            hist[z] = hist.get(z, 0.0) + tasks
            continue
        full, rem = divmod(per, short_max)
        if full:
            hist[short_max] = hist.get(short_max, 0.0) + full * nlanes / 2
        if rem >= 1:
            z = 1 << int(math.log2(rem))
            hist[z] = hist.get(z, 0.0) + nlanes / 2
    return hist


def prefix_table(rank, order, primes_mask, zs):
    """Per prefix k (1..len(order)) and segment size z: survivors and primes per position,
    and rounds per task, from the domain's ranks (primes counted for the prefixes no shorter
    than the one primes_mask was made for)."""
    L, npos = rank.shape
    n = len(order)
    ks = np.arange(1, n + 1)
    pos = L * npos
    # survivors of prefix k: positions with rank >= k
    hist = np.bincount(rank.ravel(), minlength=n + 1)
    surv = pos - np.cumsum(hist)[:n]                      # index k-1 -> rank >= k
    ph = np.bincount(rank.ravel()[primes_mask.ravel()], minlength=n + 1)
    primes = int(primes_mask.sum()) - np.cumsum(ph)[:n]
    out = {"k": ks, "surv_per_pos": surv / pos, "primes_per_pos": primes / pos, "rounds": {}}
    for z in zs:
        pairs = rank[: L - (L % 2)].reshape(L // 2, 2, npos)
        segs = pairs[:, :, : (npos // z) * z].reshape(L // 2, 2, npos // z, z)
        mx = segs.max(axis=(1, 3)).ravel()                 # max rank over the task's positions
        # rounds for prefix k: all dead -> ceil((mx + 1)/32); else every round of the prefix
        mh = np.bincount(np.minimum(mx, n), minlength=n + 1)
        cnt_dead_upto = np.cumsum(mh)                       # tasks with mx <= i
        r_of = (np.arange(n + 1) // 32 + 1).astype(np.float64)
        sum_r_dead = np.cumsum(mh * r_of)                   # sum of rounds of tasks with mx <= i
        tasks = len(mx)
        dead = cnt_dead_upto[ks - 1]                        # mx < k
        rounds = sum_r_dead[ks - 1] + (tasks - dead) * np.ceil(ks / 32)
        out["rounds"][z] = rounds / tasks
    return out


def model_terms(pt, hist, positions, idx):
    """(tasks, rounds, survivors, primes) of a batch for prefix index idx."""
    tasks = sum(hist.values())
    rounds = sum(t * pt["rounds"][z][idx] for z, t in hist.items())
    return tasks, rounds, positions * pt["surv_per_pos"][idx], positions * pt["primes_per_pos"][idx]


# ------------------------------------------------------------------ table files

def table_text(filters, header):
    body = "".join("FILTER %d %d %s\n" % f for f in filters)
    digest = hashlib.sha256(body.encode()).hexdigest()
    head = "".join("# %s\n" % h for h in header) + "# sha256=%s filters=%d\n" % (digest, len(filters))
    return head + body, digest


def build(args):
    M = args.wheel
    lanes = wheel_lanes(M)
    cands = candidates(args.mmax, M)
    groups, dens = stride_groups(cands, M, lanes)
    order = sorted(groups, key=lambda s: (-dens[s], s))
    # strides whose masks fit the budget, in density order (a stride past it would be walked
    # filter by filter): a prefix of this list is a candidate table
    fit, words = [], 0
    for s in order:
        if words + mask_words(s) <= MASK_WORDS_MAX and len(fit) < SMD_MAX:
            fit.append(s)
            words += mask_words(s)
    domains = []
    for lo in args.anchors:
        rank, kbase = first_kill_ranks(fit, groups, M, lanes, lo, args.npos)
        # primes among the positions that the shortest prefix considered leaves alive (a
        # position killed by a stride of that prefix is not a survivor of any longer one)
        primes_mask = np.zeros(rank.shape, dtype=bool)
        for li, j in np.argwhere(rank >= args.kmin):
            primes_mask[li, j] = is_prime(int(lanes[li]) + M * int(kbase[li] + j))
        domains.append((rank, primes_mask))
    return M, lanes, groups, dens, fit, domains


def averaged_prefix_table(domains, fit, zs):
    """prefix_table of each domain, averaged (equal weights: log-uniform heights)."""
    pts = [prefix_table(rank, fit, pm, zs) for rank, pm in domains]
    out = {"k": pts[0]["k"], "rounds": {}}
    for key in ("surv_per_pos", "primes_per_pos"):
        out[key] = sum(p[key] for p in pts) / len(pts)
    for z in zs:
        out["rounds"][z] = sum(p["rounds"][z] for p in pts) / len(pts)
    return out


def filters_of(strides, groups):
    out = []
    for s in strides:
        out.extend((f[0], f[1], f[2]) for f in groups[s])
    # F1 then F2, each by (mod, res): the order does not matter to the engine's results
    return sorted(out, key=lambda f: (f[2], f[0], f[1]))


def measure(paths, ks, out, steps=10):
    """Per-kernel device time of the 4096-window batch under each table (GPU): the mean of
    `steps` synchronous es_run_batch calls (es_timing, CUDA events), with a 256 MB write before
    each call to flush L2 when torch is present. Writes the calibration file --calibrate reads."""
    import es_sieve
    import workloads
    try:
        import torch
        buf = torch.empty(64 << 20, dtype=torch.int32, device="cuda:0")

        def flush():
            buf.add_(1)
            torch.cuda.synchronize()
    except Exception:
        def flush():
            pass
    wins = workloads.batch_windows(4096)
    sched = {"short_max": 64, "rung_blocks_per_sm": 4, "long_split": 1}
    rows = []
    for k, path in zip(ks, paths):
        mods, ress = es_sieve.load_filters(path)
        with es_sieve.Engine(wheel=M_DEFAULT, filters=(mods, ress), device=0) as eng:
            eng.set_schedule(**sched)
            for _ in range(3):
                eng.run_batch(wins, records=False)
            acc = {"mark_short_ms": 0.0, "mr_ms": 0.0, "rung_ms": 0.0}
            for _ in range(steps):
                flush()
                eng.run_batch(wins, records=False)
                t = eng.timing()
                for key in acc:
                    acc[key] += t[key]
            rows.append(dict({key: v / steps for key, v in acc.items()}, k=k, survivors=int(t["survivors"]),
                             primes=int(t["primes"])))
            print(json.dumps(rows[-1]), flush=True)
    json.dump({"workload": "batch4096 (workloads.batch_windows(4096)) under each prefix table", "schedule": sched,
               "timing": "es_timing per-kernel CUDA-event times, mean of %d synchronous es_run_batch calls" % steps,
               "rows": rows}, open(out, "w"), indent=1)


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--wheel", type=int, default=M_DEFAULT)
    ap.add_argument("--mmax", type=int, default=2000)
    ap.add_argument("--anchors", default=",".join(str(a) for a in ANCHORS),
                    type=lambda t: [int(x) for x in t.split(",")])
    ap.add_argument("--npos", type=int, default=NPOS)
    ap.add_argument("--kmin", type=int, default=32, help="shortest prefix modelled")
    ap.add_argument("--prefixes", default="", help="write the tables of these prefix lengths")
    ap.add_argument("--out", default=".")
    ap.add_argument("--calibrate", default="", help="JSON of measured batch timings per prefix")
    ap.add_argument("--measure", default="", help="time the --prefixes tables on the GPU, write this JSON")
    ap.add_argument("--measure-steps", type=int, default=10, help="timed calls per table for --measure")
    ap.add_argument("--write", default="", help="write the tuned table here")
    ap.add_argument("--report", action="store_true")
    ap.add_argument("--compare", default="", help="a filter table file to report on the same domains")
    args = ap.parse_args()
    import workloads
    M, lanes, groups, dens, fit, domains = build(args)
    hist = segment_histogram(workloads.batch_windows(4096), M, len(lanes))
    positions = sum(hi - lo for lo, hi in workloads.batch_windows(4096)) * len(lanes) / M
    pt = averaged_prefix_table(domains, fit, sorted(hist))
    if args.report:
        print("candidates %d, strides %d, strides within the mask budget %d" %
              (sum(len(v) for v in groups.values()), len(groups), len(fit)))
        for k in (32, 64, 96, 128, 160, 192, 224, 256, len(fit)):
            if k <= len(fit):
                t = model_terms(pt, hist, positions, k - 1)
                print("k=%3d filters=%5d surv/pos=%.3e primes/pos=%.3e rounds/task=%.3f" %
                      (k, len(filters_of(fit[:k], groups)), pt["surv_per_pos"][k - 1], pt["primes_per_pos"][k - 1],
                       t[1] / t[0]))
    if args.compare:
        tab = [(int(t[1]), int(t[2]), t[3] if len(t) > 3 else "F1")
               for t in (ln.split() for ln in open(args.compare)) if t and t[0] == "FILTER"]
        g2, d2 = stride_groups(tab, M, lanes)
        o2 = sorted(g2, key=lambda s: (-d2[s], s))
        doms = []
        for lo in args.anchors:
            rank, kbase = first_kill_ranks(o2, g2, M, lanes, lo, args.npos)
            pm = np.zeros(rank.shape, dtype=bool)
            for li, j in np.argwhere(rank >= len(o2)):
                pm[li, j] = is_prime(int(lanes[li]) + M * int(kbase[li] + j))
            doms.append((rank, pm))
        p2 = averaged_prefix_table(doms, o2, sorted(hist))
        t = model_terms(p2, hist, positions, len(o2) - 1)
        print("%s: strides=%d filters=%d surv/pos=%.3e primes/pos=%.3e rounds/task=%.3f" %
              (os.path.basename(args.compare), len(o2), len(tab), p2["surv_per_pos"][-1], p2["primes_per_pos"][-1],
               t[1] / t[0]))
    written = []
    for k in [int(x) for x in args.prefixes.split(",") if x]:
        fl = filters_of(fit[:k], groups)
        text, digest = table_text(fl, ["GB300 candidate table: the %d densest strides within the mask budget, "
                                       "every certified filter of each" % k,
                                       "M=%d mmax=%d anchors=%s npos=%d" % (M, args.mmax, ",".join("%g" % a for a in args.anchors), args.npos)])
        path = os.path.join(args.out, "f_M%d_mmax%d_gb300_k%d.txt" % (M, args.mmax, k))
        open(path, "w").write(text)
        written.append((k, path))
        print(path, digest)
    if args.measure:
        measure([p for _, p in written], [k for k, _ in written], args.measure, args.measure_steps)
    if args.calibrate:
        # [{"k": k, "mark_short_ms": .., "mr_ms": .., "rung_ms": ..}, ...] of one batch per prefix
        meas = json.load(open(args.calibrate))
        meas = meas["rows"] if isinstance(meas, dict) else meas
        terms = {i: model_terms(pt, hist, positions, i) for i in range(len(fit))}
        coef = {}
        for key, col in (("mark_short_ms", 1), ("mr_ms", 2), ("rung_ms", 3)):
            x = np.array([terms[row["k"] - 1][col] for row in meas])
            y = np.array([row[key] for row in meas])
            A = np.stack([np.ones_like(x), x], axis=1)
            (c0, c1), *_ = np.linalg.lstsq(A, y, rcond=None)
            coef[key] = (float(c0), float(max(c1, 0.0)))
            print("%-14s = %.4f + %.4e * %s" % (key, c0, c1, ("rounds", "survivors", "primes")[col - 1]))

        def modelled(i):
            t = terms[i]
            return sum(coef[key][0] + coef[key][1] * t[col]
                       for key, col in (("mark_short_ms", 1), ("mr_ms", 2), ("rung_ms", 3)))
        for row in meas:
            print("k=%3d measured %.4f ms, modelled %.4f ms" %
                  (row["k"], row["mark_short_ms"] + row["mr_ms"] + row["rung_ms"], modelled(row["k"] - 1)))
        lo = max(args.kmin, 1) - 1
        best = min(range(lo, len(fit)), key=modelled) + 1
        print("best prefix k=%d, modelled %.4f ms per batch" % (best, modelled(best - 1)))
        if args.write:
            fl = filters_of(fit[:best], groups)
            text, digest = table_text(fl, [
                "certified filter table tuned for the GB300 engine's kill-mask marking (filter_tune.py)",
                "every certified candidate (F1 m <= mmax, F2 r <= 63 u <= 64; modulus not dividing M) of the",
                "%d densest strides whose masks fit the per-lane budget" % best,
                "M=%d mmax=%d anchors=%s npos=%d" % (M, args.mmax, ",".join("%g" % a for a in args.anchors), args.npos),
                "k_mark_short_ms=%.4f+%.4e*rounds k_mr_ms=%.4f+%.4e*survivors k_rung_ms=%.4f+%.4e*primes" %
                (coef["mark_short_ms"] + coef["mr_ms"] + coef["rung_ms"])])
            open(args.write, "w").write(text)
            print(args.write, digest)

if __name__ == "__main__":
    main()
