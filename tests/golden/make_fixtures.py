"""Regenerate the golden fixtures in tests/golden/ from the reference tree.

Run with REF set to the reference tree, after `make -C oracle ref REF=...` built the
reference scanners into oracle/_ref/ (`python -c "import __graft_entry__ as g; g.build()"`
does both where the tree is present). Two kinds of fixture:

  copied    data the reference ships for this path, byte for byte: its filter tables
            (tables/filters/), the decade windows (data/rederive/decades/), the w19 window's
            complete certificate set and the w64 window's SUMMARY, head, tail and stream
            digests (data/rederive/windows/), the 10^15 shard SUMMARYs
            (data/sieve15/SUMMARY.txt), and the sha256 of both class tables
            (tables/class_table_*.txt)
  generated outputs of the reference scanners built from its own sources (rung_scan3,
            cover_scan, and ref_sweep over rung_scan3's sweep_lane), on the seeded
            configurations of erdos-strauss_gb300/workloads.py and the rows of the
            reference's differential gate (tests/diff3.sh, Makefile:79-103)

  python tests/golden/make_fixtures.py [--only NAME ...]
      NAME: copied, rows (the CLI and sweep rows), batch (the 4096-window batch, every
      window's SUMMARY and record digest), batch19 (the same at the top of the range);
      default all. MANIFEST.txt keeps the entries of the fixtures not regenerated.

The GPU tests and the CPU oracle tests read only these files; nothing at run time needs the
reference tree.
"""
import argparse
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("REF", "")
BIN = os.path.join(ROOT, "oracle", "_ref")
sys.path.insert(0, os.path.join(ROOT, "erdos-strauss_gb300"))
import workloads  # noqa: E402

FILTERS = ["f_M120120_mmax2000_runtime.txt", "f_M2042040_mmax2000_gpu.txt", "f_M2042040_mmax2000_runtime.txt"]
GPU = "f_M2042040_mmax2000_gpu.txt"
# the table tuned for the GB300 engine (erdos-strauss_gb300/filter_tune.py): not the reference's,
# so its fixtures are the reference's scanner run on it, never a copied golden
GB300_TABLE = os.path.join(os.path.dirname(os.path.dirname(HERE)), "erdos-strauss_gb300", "tables",
                           "f_M2042040_mmax2000_gb300.txt")


def sha256(path):
    h = hashlib.sha256()
    with open(path, "rb") as f:
        for blk in iter(lambda: f.read(1 << 20), b""):
            h.update(blk)
    return h.hexdigest()


def run(args, out):
    r = subprocess.run(args, capture_output=True)
    if r.returncode not in (0, 2):
        raise SystemExit("failed: %s\n%s" % (" ".join(args), r.stderr.decode()))
    with open(out, "wb") as f:
        f.write(r.stdout)
    return r.returncode


def write_windows(path, wins):
    with open(path, "w") as f:
        for a, b in wins:
            f.write("%d %d\n" % (a, b))


def window_digests(sweep, wfile, table, out):
    """Every window of a batch through the reference's sweep_lane (ref_sweep --windows), kept
    as one line per window: the sha256 of its record lines (certificates and SURVIVORs, in the
    reference's lane-major order), their count, and its SUMMARY line."""
    p = subprocess.Popen([sweep, "--windows", wfile, "--filters", table], stdout=subprocess.PIPE)
    h, n, lines = hashlib.sha256(), 0, []
    for ln in p.stdout:
        if ln.startswith(b"SUMMARY "):
            lines.append("%s %d %s" % (h.hexdigest(), n, ln.decode()))
            h, n = hashlib.sha256(), 0
        else:
            h.update(ln)
            n += 1
    if p.wait() not in (0, 2):
        raise SystemExit("ref_sweep failed on " + wfile)
    with open(out, "w") as f:
        f.write("".join(lines))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", nargs="*", default=["copied", "rows", "batch", "batch19", "gb300"])
    args = ap.parse_args()
    if not REF or not os.path.isdir(REF) or not os.path.exists(os.path.join(BIN, "rung_scan3")):
        raise SystemExit("set REF to the reference tree and build oracle/_ref (make -C oracle ref REF=...)")
    for d in ("filters", "decades", "windows", "gen", "metas"):
        os.makedirs(os.path.join(HERE, d), exist_ok=True)
    manifest = {}                 # fixture -> "sha256 generator args" (kept for what is not redone)
    mpath = os.path.join(HERE, "MANIFEST.txt")
    if os.path.exists(mpath):
        for ln in open(mpath):
            if not ln.startswith("#") and ln.strip():
                k, rest = ln.rstrip("\n").split(" ", 1)
                manifest[k] = rest
    rows = []   # (file, generator, argv after the binary) -- the file holds the binary's stdout
    rs3, cov, sweep = (os.path.join(BIN, b) for b in ("rung_scan3", "cover_scan", "ref_sweep"))
    F = {f: os.path.join(HERE, "filters", f) for f in FILTERS}
    gen = os.path.join(HERE, "gen")

    def cli(name, binary, *a):
        run([binary] + [str(x) for x in a], os.path.join(gen, name))
        rows.append((name, os.path.basename(binary), [str(x) for x in a]))

    if "copied" in args.only:
        for f in FILTERS:
            shutil.copyfile(os.path.join(REF, "tables", "filters", f), os.path.join(HERE, "filters", f))
        for k in range(6, 20):
            shutil.copyfile(os.path.join(REF, "data", "rederive", "decades", "d%d.txt" % k),
                            os.path.join(HERE, "decades", "d%d.txt" % k))
        for f in ("w19_certificates.txt", "w64_summary.txt", "w64_head.txt", "w64_tail.txt", "w64.sha256"):
            shutil.copyfile(os.path.join(REF, "data", "rederive", "windows", f), os.path.join(HERE, "windows", f))
        shutil.copyfile(os.path.join(REF, "data", "sieve15", "SUMMARY.txt"), os.path.join(HERE, "sieve15_SUMMARY.txt"))
        shutil.copyfile(os.path.join(REF, "data", "c19", "shard_0.meta"), os.path.join(HERE, "metas", "c19_shard_0.meta"))
        with open(os.path.join(HERE, "class_tables.sha256"), "w") as f:
            for M in (120120, 2042040):
                f.write("%s  class_table_%d.txt\n" % (sha256(os.path.join(REF, "tables", "class_table_%d.txt" % M)), M))
    if "rows" in args.only:
        c1 = workloads.c1()
        cli("c1_runtime.out", rs3, c1["lo"], c1["hi"], "--wheel", 120120, "--filters", F[c1["filters"]])
        cli("c1_default.out", rs3, c1["lo"], c1["hi"], "--wheel", 120120)
        cli("c1_default_cover_scan.out", cov, c1["lo"], c1["hi"], "--wheel", 120120)
        for cfg in (workloads.c2(), workloads.c3()):
            cli("%s_gpu.out" % cfg["name"], sweep, cfg["lo"], cfg["hi"], "--filters", F[GPU])
        c2 = workloads.c2()
        cli("c2_runtime.out", sweep, c2["lo"], c2["hi"], "--filters", F["f_M2042040_mmax2000_runtime.txt"])
        # the differential gate's rows (Makefile:79-82), and their --seg / --sieve / shard variants
        lo, hi = 1000000000000, 1000200000000
        cli("d3_120120_m200.out", rs3, lo, hi, "--wheel", 120120, "--mmax", 200)
        cli("d3_120120_m200_cover_scan.out", cov, lo, hi, "--wheel", 120120, "--mmax", 200)
        cli("d3_120120_m200_sieve1000.out", rs3, lo, hi, "--wheel", 120120, "--mmax", 200, "--sieve", 1000)
        for i in range(4):
            cli("d3_120120_m200_shard%d_4.out" % i, rs3, lo, hi, "--wheel", 120120, "--mmax", 200, "--shard", "%d/4" % i)
        cli("d3_120120_m2000.out", rs3, lo, 1000010000000, "--wheel", 120120, "--mmax", 2000)
        cli("d3_2042040_m200.out", rs3, lo, hi, "--wheel", 2042040, "--mmax", 200)
        cli("d3_2042040_m200_nosurv.out", rs3, lo, hi, "--wheel", 2042040, "--mmax", 200, "--no-emit-survivors")
        # stage E inside a scan: cover_scan's test hook skips stage D (sieve/cover_scan.cpp:395,
        # :431), so every prime goes to the direct search and the unsolved ones are SURVIVORs
        cli("d3_120120_m200_norung_cover_scan.out", cov, lo, hi, "--wheel", 120120, "--mmax", 200, "--no-rung")
        # top of the range: the last 2^32 integers below the stage-E ceiling, pruned table plus
        # stage B' primes
        top = workloads.DIRECT_PMAX
        cli("top_gpu_sieve500.out", sweep, top - (1 << 32), top, "--filters", F[GPU], "--sieve", 500)
        # stage E either side of 2^63 (Makefile:98-103)
        for h in (9223372036854770000, 9223372036854775808, 9999999999999990000, 18446744065119000000):
            cli("direct_%d.out" % h, rs3, "--check-direct", h, 20)
        # a sample of the batched configuration: its first 48 windows, each through sweep_lane
        wf = os.path.join(gen, "batch48.windows")
        write_windows(wf, workloads.batch_windows()[:48])
        cli("batch48.out", sweep, "--windows", wf, "--filters", F[GPU])
    # whole batches: the exact windows, and per window the digest of its records and its SUMMARY
    for key, name, wins in (("batch", "batch4096", workloads.batch_windows),
                            ("batch19", "batch19_4096", workloads.batch19_windows)):
        if key not in args.only:
            continue
        wf = os.path.join(gen, name + ".windows")
        write_windows(wf, wins(4096))
        rows.append((name + ".windows", "workloads.%s" % wins.__name__, ["4096"]))
        window_digests(sweep, wf, F[GPU], os.path.join(gen, name + ".digests"))
        rows.append((name + ".digests", "ref_sweep", ["--windows", wf, "--filters", F[GPU]]))
    if "gb300" in args.only:
        # the tuned table through the reference's sweep_lane: the mid-height and top-of-range
        # shards, and both batches window by window
        for cfg in (workloads.c2(), workloads.c3()):
            cli("%s_gb300.out" % cfg["name"], sweep, cfg["lo"], cfg["hi"], "--filters", GB300_TABLE)
        for name in ("batch4096", "batch19_4096"):
            wf = os.path.join(gen, name + ".windows")
            window_digests(sweep, wf, GB300_TABLE, os.path.join(gen, name + "_gb300.digests"))
            rows.append((name + "_gb300.digests", "ref_sweep", ["--windows", wf, "--filters", GB300_TABLE]))
    for name, binary, a in rows:
        rel = [os.path.relpath(x, HERE) if x.startswith(ROOT) else x for x in a]
        manifest["gen/" + name] = "%s %s %s" % (sha256(os.path.join(gen, name)), binary, " ".join(rel))
    for d in ("filters", "decades", "windows", "metas"):
        for name in sorted(os.listdir(os.path.join(HERE, d))):
            if name.startswith("gb300_"):
                continue          # written by this engine on a GB300, not copied: its entry stays
            manifest["%s/%s" % (d, name)] = "%s copied" % sha256(os.path.join(HERE, d, name))
    manifest["sieve15_SUMMARY.txt"] = "%s copied" % sha256(os.path.join(HERE, "sieve15_SUMMARY.txt"))
    with open(mpath, "w") as f:
        f.write("# fixture  sha256  generator and arguments (paths relative to tests/golden)\n")
        for k in sorted(manifest, key=lambda k: (not k.startswith("gen/"), k)):
            f.write("%s %s\n" % (k, manifest[k]))
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
