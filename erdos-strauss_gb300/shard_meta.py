"""Shard records (metas) of the production sieve: parse, write through the GB300 CLI, audit.

A meta is the durable record of one shard (tools/run19.sh:70-77): a provenance header,
`certs=` (RUNG and SOLVED lines), `cert_sha256=` (sha256 of the certificate stream, every
line but SUMMARY, in emission order), SURVIVOR lines verbatim, and the SUMMARY line last.
`rung_scan3_gb300 LO HI --shard i/N --filters T --meta FILE` writes one on the GPU; this
module reads them (the rules of sieve/shard_meta.py:25-60) and compares two.

Emission order: the production driver emits rounds of --seg positions, lanes in wheel order
within a round (sieve/cuda/scan.cu:266-310); rung_scan3 emits lane by lane. `round_order`
rearranges a lane-major stream into round order, so either digest can be recomputed from the
other's text.
"""
import hashlib
import re
import subprocess

HERE = __import__("os").path.dirname(__import__("os").path.abspath(__file__))
CLI = __import__("os").path.join(HERE, "rung_scan3_gb300")
HDR = re.compile(r"# shard (\d+)/(\d+)\s+rc=(-?\d+)\s+wall=(\d+)s\s+attempt=(\d+)\s+(.*)")


def parse_meta(text):
    """One meta's text -> dict: header fields, certs, cert_sha256, survivor_lines, the
    SUMMARY fields, and complete (SUMMARY seen)."""
    d = {"survivor_lines": [], "complete": False}
    for line in text.splitlines():
        line = line.strip()
        if not line:
            continue
        m = HDR.match(line)
        if m:
            d.update(idx=int(m.group(1)), nshards=int(m.group(2)), rc=int(m.group(3)), wall=int(m.group(4)),
                     attempt=int(m.group(5)))
        elif line.startswith("# "):
            for kv in line[2:].split():
                k, _, v = kv.partition("=")
                if k:
                    d[k] = int(v) if v.isdigit() else v
        elif line.startswith("SURVIVOR"):
            d["survivor_lines"].append(line)
        elif line.startswith("SUMMARY"):
            d["summary"] = line
            for kv in line.split()[1:]:
                k, _, v = kv.partition("=")
                d[k] = int(v) if v.isdigit() else v
            d["complete"] = True
        elif "=" in line:
            k, _, v = line.partition("=")
            d[k] = int(v) if v.isdigit() else v
    if "mr" in d and "composite" in d:
        d["primes"] = d["mr"] - d["composite"]
    return d


def audit(a, b, compare_digest=True):
    """Differences between two parsed metas of the same shard: SUMMARY, certs, survivors
    and (when both used the same emission order) cert_sha256. Empty list = they agree."""
    bad = []
    if not (a.get("complete") and b.get("complete")):
        bad.append("incomplete meta (no SUMMARY)")
    if a.get("summary") != b.get("summary"):
        bad.append("SUMMARY differs")
    if a.get("certs") != b.get("certs"):
        bad.append("certs %s != %s" % (a.get("certs"), b.get("certs")))
    if a.get("survivor_lines") != b.get("survivor_lines"):
        bad.append("SURVIVOR lines differ")
    if compare_digest and a.get("cert_sha256") != b.get("cert_sha256"):
        bad.append("cert_sha256 differs")
    return bad


def round_order(text, lo, M, classes, seg):
    """A lane-major certificate stream for [lo, hi) (SUMMARY excluded) in the production
    driver's order: key (J // seg, lane, J) with J the line's position index in its lane."""
    lane_of = {c: i for i, c in enumerate(classes)}
    keyed = []
    for n, line in enumerate(text.splitlines(keepends=True)):
        p = int(line.split()[1])
        rho = p % M
        first = lo + (rho - lo) % M
        J = (p - first) // M
        keyed.append(((J // seg, lane_of[rho], J, n), line))
    keyed.sort()
    return "".join(line for _, line in keyed)


def stream_digest(text):
    """certs= and cert_sha256= of a certificate stream (SUMMARY lines dropped)."""
    body = "".join(ln for ln in text.splitlines(keepends=True) if not ln.startswith("SUMMARY "))
    certs = sum(1 for ln in body.splitlines() if ln.startswith(("RUNG ", "SOLVED ")))
    return certs, hashlib.sha256(body.encode()).hexdigest()


def write_meta(path, lo, hi, filters=None, shard=None, order="round", seg=262144, chunk_rounds=64, wheel=2042040,
               extra=()):
    """Run the GB300 CLI for one shard and write its meta; returns (exit code, parsed meta)."""
    cmd = [CLI, str(lo), str(hi), "--wheel", str(wheel), "--seg", str(seg), "--meta", path, "--order", order,
           "--chunk-rounds", str(chunk_rounds)]
    if filters:
        cmd += ["--filters", filters]
    if shard:
        cmd += ["--shard", "%d/%d" % shard]
    r = subprocess.run(cmd + list(extra), capture_output=True, text=True)
    if r.returncode not in (0, 2):
        raise RuntimeError("rung_scan3_gb300 failed (%d): %s" % (r.returncode, r.stderr[-500:]))
    with open(path) as f:
        return r.returncode, parse_meta(f.read())
