"""Regenerate the golden fixtures in tests/golden/ from the reference tree.

Run in a container that has the reference at REF (default /root/reference) after
`make -C oracle ref` built the reference scanners into oracle/_ref/. Two kinds of fixture:

  copied    data the reference ships for this path, byte for byte: its filter tables
            (tables/filters/), the decade windows (data/rederive/decades/), the w19 window's
            complete certificate set and the w64 window's SUMMARY, head and tail
            (data/rederive/windows/), the 10^15 shard SUMMARYs (data/sieve15/SUMMARY.txt),
            and the sha256 of both class tables (tables/class_table_*.txt)
  generated outputs of the reference scanners built from its own sources (rung_scan3,
            cover_scan, and ref_sweep over rung_scan3's sweep_lane), on the seeded
            configurations of erdos-strauss_gb300/workloads.py and the rows of the
            reference's differential gate (tests/diff3.sh, Makefile:79-103)

The GPU tests and the CPU oracle tests read only these files; nothing at run time needs the
reference tree.
"""
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("REF", "/root/reference")
BIN = os.path.join(ROOT, "oracle", "_ref")
sys.path.insert(0, os.path.join(ROOT, "erdos-strauss_gb300"))
import workloads  # noqa: E402

FILTERS = ["f_M120120_mmax2000_runtime.txt", "f_M2042040_mmax2000_gpu.txt", "f_M2042040_mmax2000_runtime.txt"]


def sha256(path):
    return hashlib.sha256(open(path, "rb").read()).hexdigest()


def run(args, out):
    r = subprocess.run(args, capture_output=True)
    if r.returncode not in (0, 2):
        raise SystemExit("failed: %s\n%s" % (" ".join(args), r.stderr.decode()))
    with open(out, "wb") as f:
        f.write(r.stdout)
    return r.returncode


def main():
    if not os.path.isdir(REF) or not os.path.exists(os.path.join(BIN, "rung_scan3")):
        raise SystemExit("needs the reference tree and `make -C oracle ref`")
    os.makedirs(os.path.join(HERE, "filters"), exist_ok=True)
    os.makedirs(os.path.join(HERE, "decades"), exist_ok=True)
    os.makedirs(os.path.join(HERE, "windows"), exist_ok=True)
    os.makedirs(os.path.join(HERE, "gen"), exist_ok=True)
    # ---- copied
    for f in FILTERS:
        shutil.copyfile(os.path.join(REF, "tables", "filters", f), os.path.join(HERE, "filters", f))
    for k in range(6, 20):
        shutil.copyfile(os.path.join(REF, "data", "rederive", "decades", "d%d.txt" % k),
                        os.path.join(HERE, "decades", "d%d.txt" % k))
    for f in ("w19_certificates.txt", "w64_summary.txt", "w64_head.txt", "w64_tail.txt"):
        shutil.copyfile(os.path.join(REF, "data", "rederive", "windows", f), os.path.join(HERE, "windows", f))
    shutil.copyfile(os.path.join(REF, "data", "sieve15", "SUMMARY.txt"), os.path.join(HERE, "sieve15_SUMMARY.txt"))
    os.makedirs(os.path.join(HERE, "metas"), exist_ok=True)
    shutil.copyfile(os.path.join(REF, "data", "c19", "shard_0.meta"), os.path.join(HERE, "metas", "c19_shard_0.meta"))
    with open(os.path.join(HERE, "class_tables.sha256"), "w") as f:
        for M in (120120, 2042040):
            f.write("%s  class_table_%d.txt\n" % (sha256(os.path.join(REF, "tables", "class_table_%d.txt" % M)), M))
    # ---- generated by the reference scanners
    rs3, cov, sweep = (os.path.join(BIN, b) for b in ("rung_scan3", "cover_scan", "ref_sweep"))
    F = {f: os.path.join(HERE, "filters", f) for f in FILTERS}
    gen = os.path.join(HERE, "gen")
    rows = []   # (file, argv after the binary) -- the file holds the binary's stdout

    def cli(name, binary, *args):
        run([binary] + [str(a) for a in args], os.path.join(gen, name))
        rows.append((name, os.path.basename(binary), [str(a) for a in args]))

    c1 = workloads.c1()
    cli("c1_runtime.out", rs3, c1["lo"], c1["hi"], "--wheel", 120120, "--filters", F[c1["filters"]])
    cli("c1_default.out", rs3, c1["lo"], c1["hi"], "--wheel", 120120)
    cli("c1_default_cover_scan.out", cov, c1["lo"], c1["hi"], "--wheel", 120120)
    for cfg in (workloads.c2(), workloads.c3()):
        cli("%s_gpu.out" % cfg["name"], sweep, cfg["lo"], cfg["hi"], "--filters", F["f_M2042040_mmax2000_gpu.txt"])
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
    cli("top_gpu_sieve500.out", sweep, top - (1 << 32), top, "--filters", F["f_M2042040_mmax2000_gpu.txt"],
        "--sieve", 500)
    # stage E either side of 2^63 (Makefile:98-103)
    for h in (9223372036854770000, 9223372036854775808, 9999999999999990000, 18446744065119000000):
        cli("direct_%d.out" % h, rs3, "--check-direct", h, 20)
    # a sample of the batched configuration: its first 48 windows, each through sweep_lane
    wins = workloads.batch_windows()[:48]
    wf = os.path.join(gen, "batch48.windows")
    with open(wf, "w") as f:
        for a, b in wins:
            f.write("%d %d\n" % (a, b))
    cli("batch48.out", sweep, "--windows", wf, "--filters", F["f_M2042040_mmax2000_gpu.txt"])
    with open(os.path.join(HERE, "MANIFEST.txt"), "w") as f:
        f.write("# fixture  sha256  generator and arguments (paths relative to tests/golden)\n")
        for name, binary, args in rows:
            rel = [os.path.relpath(a, HERE) if a.startswith(HERE) else a for a in args]
            f.write("gen/%s %s %s %s\n" % (name, sha256(os.path.join(gen, name)), binary, " ".join(rel)))
        for d in ("filters", "decades", "windows", "metas"):
            for name in sorted(os.listdir(os.path.join(HERE, d))):
                f.write("%s/%s %s copied\n" % (d, name, sha256(os.path.join(HERE, d, name))))
        for name in ("sieve15_SUMMARY.txt",):
            f.write("%s %s copied\n" % (name, sha256(os.path.join(HERE, name))))
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
