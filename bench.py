#!/usr/bin/env python3
"""Throughput of the GB300 verification-sieve engine: verified integers/s on one GB300.

Workload (default `batch`): the batched configuration -- 4096 windows of lengths
floor(2^(16 + 12 U)) and log-uniform start heights over [255255, 1.8446744065e19], seeded
splitmix64 (erdos-strauss_gb300/workloads.py), wheel 2042040, the pruned gpu filter table.
One step = one pass of the whole funnel (marking, compaction, Miller-Rabin, rung walk, direct
search) over every window of the batch, through es_run_batch with the persistent schedule,
records and counters returned to the host. Before the warm-up, es_autotune picks the kernel
schedule on the same batch (untimed; every schedule gives identical results).

  value   integers of the batch / device time of the step's kernels (CUDA events on the
          engine's stream, inputs already resident; L2 flushed before every timed step)
  e2e     the same integers / wall time of the es_run_batch call from host buffers
          (window list in, counters and sorted binary records out)
  plain   the same windows through per-window launches of the same kernels
  c3      one 2^34-integer window at height >= 1.7e19, plain launch (the "at 1e19" row)
  serve   2000 single-window requests arriving as a Poisson stream through es_submit/es_poll
          (continuous batching over two streams): p50/p99 latency and integers/s

--impl reference times the reference algorithm on the host cores (the CPU oracle port, all
threads) on a bounded sample of the same workload. Multi-GPU: one process per GPU under
torchrun, each rank its own seeded batch (weak scaling); value = all ranks' integers / the
slowest rank's time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "erdos-strauss_gb300"))
import workloads  # noqa: E402

GOLDEN = os.path.join(ROOT, "tests", "golden")
GPU_TABLE = os.path.join(GOLDEN, "filters", "f_M2042040_mmax2000_gpu.txt")
# the filter table tuned for this engine (erdos-strauss_gb300/filter_tune.py; its own digest,
# never the parity default): reported beside the reference's table
GB300_TABLE = os.path.join(ROOT, "erdos-strauss_gb300", "tables", "f_M2042040_mmax2000_gb300.txt")
METRIC = "verified integers/s at 1e19 (batched vs plain, 1 GB300)"
# One ncu capture per kernel schedule of the 4096-window batch with the gpu table (the
# profiles/ summaries give the commands): per launch, the warp instructions
# (smsp__inst_executed.sum) and DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum).
# k_mark_short's depend on (short_max, long_split), k_rung's on rung_blocks_per_sm. A schedule
# with no capture here gets no issue figure rather than another schedule's.
MARK_SHORT_NCU = {            # (short_max, long_split) -> per launch
    (32, 1): {"inst": 728342167, "dram": 95922688 + 3819776},
    (64, 1): {"inst": 718216590, "dram": 95236608 + 3364864},
    (128, 1): {"inst": 735127673, "dram": 95047680 + 3439104},
}
RUNG_NCU = {                  # rung_blocks_per_sm -> per launch
    4: {"inst": 70295758, "dram": 845824 + 768},
    6: {"inst": 70433215, "dram": 845824},
    8: {"inst": 70539276, "dram": 846592},
}
# Cover/filter marks per integer of the 2042040 wheel with the gpu filter table: 9.0951 marks per
# position (positions of all 2308 lanes, all 3745 filters) over 2042040 / 2308 integers per position.
MARKS_PER_INTEGER_GPU = 9.0951 / (2042040 / 2308)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--windows", type=int, default=4096)
    ap.add_argument("--sieve", type=int, default=0, help="stage B' small primes up to P (rung_scan3 --sieve P)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--cpu-windows", type=int, default=CPU_WINDOWS,
                    help="the CPU baseline's fixed sample: this many leading windows of the batch")
    ap.add_argument("--serve", type=int, default=2000, help="serving requests (0: no serving leg)")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default schedule")
    ap.add_argument("--schedule", default="", help="short_max,rung_blocks_per_sm,long_split: set, no autotune")
    ap.add_argument("--no-batch19", action="store_true", help="skip the batch at [1e19, ceiling)")
    ap.add_argument("--no-pipelined", action="store_true",
                    help="skip the pipelined leg (for profiler runs: under ncu the process ended with a "
                         "segmentation fault when the pipelined leg started); e2e is then the synchronous figure")
    ap.add_argument("--no-tuned-table", action="store_true", help="skip the legs with the GB300-tuned filter table")
    return ap.parse_args()


def dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as td
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        td.init_process_group(backend="gloo")
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as td
        td.barrier()


def allmax(ws, v):
    if ws == 1:
        return v
    import torch
    import torch.distributed as td
    t = torch.tensor([float(v)], dtype=torch.float64)
    td.all_reduce(t, op=td.ReduceOp.MAX)
    return float(t.item())


def allsum(ws, v):
    if ws == 1:
        return v
    import torch
    import torch.distributed as td
    t = torch.tensor([float(v)], dtype=torch.float64)
    td.all_reduce(t, op=td.ReduceOp.SUM)
    return float(t.item())


class Clocks:
    """SM clock and clock-event reasons of the GPU, sampled during the timed region.

    NVML through ctypes every 2 ms (the timed region of a default run is tens of ms), falling
    back to nvidia-smi every 200 ms. The GPU is found by its PCI bus id, so the sample is of
    the device the engine runs on whatever CUDA_VISIBLE_DEVICES says. Reads only."""
    REASONS = ((0x4, "sw_power_cap"), (0x8, "hw_slowdown"), (0x20, "sw_thermal_slowdown"),
               (0x40, "hw_thermal_slowdown"), (0x80, "hw_power_brake_slowdown"))
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.busid = None
        try:
            import torch
            pr = torch.cuda.get_device_properties(device)
            self.busid = "%08X:%02X:%02X.0" % (pr.pci_domain_id, pr.pci_bus_id, pr.pci_device_id)
        except Exception:
            pass
        self.samples, self.max_mhz, self.source = [], None, None
        self.stop = None
        self.p = None

    def _nvml(self):
        import ctypes as C
        lib = C.CDLL("libnvidia-ml.so.1")
        if lib.nvmlInit_v2() != 0:
            raise OSError("nvmlInit")
        h = C.c_void_p()
        if self.busid:
            st = lib.nvmlDeviceGetHandleByPciBusId_v2(self.busid.encode(), C.byref(h))
        else:
            st = lib.nvmlDeviceGetHandleByIndex_v2(self.device, C.byref(h))
        if st != 0:
            raise OSError("nvml handle")
        return C, lib, h

    def __enter__(self):
        import threading
        try:
            C, lib, h = self._nvml()
            mx = C.c_uint()
            if lib.nvmlDeviceGetMaxClockInfo(h, 1, C.byref(mx)) == 0:
                self.max_mhz = float(mx.value)
            reasons_fn = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
                lib.nvmlDeviceGetCurrentClocksThrottleReasons
            self.stop = threading.Event()

            def loop():
                mhz, rs = C.c_uint(), C.c_ulonglong()
                while not self.stop.is_set():
                    if lib.nvmlDeviceGetClockInfo(h, 1, C.byref(mhz)) == 0 and reasons_fn(h, C.byref(rs)) == 0:
                        self.samples.append((float(mhz.value), int(rs.value)))
                    time.sleep(0.002)
            self.th = threading.Thread(target=loop, daemon=True)
            self.th.start()
            self.source = "nvml 2 ms"
        except (OSError, AttributeError):
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            try:
                self.p = subprocess.Popen(["nvidia-smi", "-i", self.busid or str(self.device),
                                           "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                                           "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
                self.source = "nvidia-smi 200 ms"
            except OSError:
                self.p = None
        return self

    def __exit__(self, *a):
        if self.stop is not None:
            self.stop.set()
            self.th.join()
        if self.p:
            self.p.terminate()
            self.p.wait()

    def _smi_rows(self):
        self.f.flush()
        rows = []
        for ln in open(self.f.name):
            t = [x.strip() for x in ln.split(",")]
            if len(t) >= 9 and t[1].replace(".", "").isdigit():
                bits = 0
                for (bit, _), val in zip(((0x8, 0), (0x40, 0), (0x20, 0), (0x4, 0)), t[5:9]):
                    if val.lower().startswith("active"):
                        bits |= bit
                rows.append((float(t[1]), bits))
                if t[2].replace(".", "").isdigit():
                    self.max_mhz = max(self.max_mhz or 0.0, float(t[2]))
        os.unlink(self.f.name)
        return rows

    def summary(self):
        rows = self.samples if self.stop is not None else (self._smi_rows() if self.p else [])
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": self.max_mhz, "reasons": ["unsampled"], "samples": 0}
        seen = 0
        for _, bits in rows:
            seen |= bits
        return {"sm_mhz": statistics.median(m for m, _ in rows), "sm_max_mhz": self.max_mhz,
                "reasons": [name for bit, name in self.REASONS if seen & bit], "samples": len(rows),
                "source": self.source}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def integers(wins):
    return sum(hi - lo for lo, hi in wins)


def l2_flusher(device):
    """A 256 MB device buffer rewritten before every timed step (larger than the 129 MB L2).
    flush() waits for the write; flush_async() only queues it (on torch's stream, which the
    engine's streams do not wait for), for the pipelined leg, where a wait would drain the
    batches in flight."""
    try:
        import torch
        buf = torch.empty(64 * 1024 * 1024, dtype=torch.int32, device="cuda:%d" % device)

        def flush_async(k=[0]):
            k[0] += 1
            buf.fill_(k[0])

        def flush():
            flush_async()
            torch.cuda.synchronize(device)
        return flush, flush_async, "flushed (256 MB write before each timed step)"
    except Exception as ex:  # torch missing: say so rather than hide it
        return (lambda: None), (lambda: None), "not flushed (%s)" % type(ex).__name__


# The CPU baseline's fixed sample: the first CPU_WINDOWS windows of the batch (8.2e9 integers
# of the seeded 4096-window batch), timed whole by both arms.
CPU_WINDOWS = 256


def host_cpu():
    """The host's CPU model, instruction set and thread count (lscpu, else /proc/cpuinfo)."""
    import platform
    info = {"isa": platform.machine(), "threads": os.cpu_count(), "model": None}
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            k, _, v = ln.partition(":")
            if k.strip() == "Model name" and v.strip():
                info["model"] = v.strip()
            if k.strip() == "Vendor ID" and v.strip():
                info["vendor"] = v.strip()
            if k.strip() == "Flags":
                fl = v.split()
                info["simd"] = [f for f in ("sse4_2", "avx2", "avx512f", "asimd", "sve", "sve2") if f in fl]
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for ln in open("/proc/cpuinfo"):
            k, _, v = ln.partition(":")
            if k.strip() == "Features" and "simd" not in info:
                fl = v.split()
                info["simd"] = [f for f in ("asimd", "sve", "sve2") if f in fl]
            if k.strip() == "model name" and not info["model"]:
                info["model"] = v.strip()
    except OSError:
        pass
    return info


def cpu_baseline(wins, seconds, threads=None):
    """The reference algorithm (CPU oracle port) on the host cores over the leading windows of
    the workload until `seconds` have elapsed. Returns (integers/s, windows done, cores)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    import es_sieve
    mods, ress = es_sieve.load_filters(GPU_TABLE)
    mods, ress = [int(m) for m in mods], [int(r) for r in ress]
    cores = threads or os.cpu_count()
    done, ints, t0 = 0, 0, time.perf_counter()
    for lo, hi in wins:
        oracle.scan(lo, hi, 2042040, mods, ress, len(mods), threads=cores)
        done += 1
        ints += hi - lo
        if time.perf_counter() - t0 > seconds:
            break
    el = time.perf_counter() - t0
    return ints / el, done, cores, el


def run_reference(args, ws, rank):
    if rank != 0:
        return
    wins = workloads.batch_windows(args.windows)
    cores = os.cpu_count()
    for _ in range(args.warmup):
        cpu_baseline(wins[:2], 0.0, cores)
    sample = wins[:args.cpu_windows]
    tot_ints, tot_s = 0, 0.0
    for k in range(args.steps):
        rate, done, _, el = cpu_baseline(sample, float("inf"), cores)
        tot_ints += rate * el
        tot_s += el
    value = tot_ints / tot_s
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "integers/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * tot_s / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64", "data": "synthetic",
            "config": {"workload": "batch4096", "windows": args.windows, "wheel": 2042040,
                       "filters": "f_M2042040_mmax2000_gpu.txt", "seed": workloads.SEED},
            "cpu_baseline": {"value": value, "unit": "integers/s", "cores": cores, "kind": "port",
                             "sample": "each step: the first %d windows of the 4096-window batch (%d integers)"
                                       % (len(sample), integers(sample)), "host": host_cpu()},
            "e2e": {"value": value, "unit": "integers/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def percentile(xs, q):
    """Nearest-rank percentile of a non-empty list."""
    ys = sorted(xs)
    return ys[min(len(ys) - 1, max(0, int(-(-q * len(ys) // 100)) - 1))]


def serve_leg(eng, n, seed):
    """Serving: n requests arriving as a Poisson stream (mean gap 0.5 ms, lengths 2^12..2^30,
    workloads.serve_requests) through es_submit / es_poll. A submitting thread keeps the arrival
    times; the main thread sweeps the outstanding tickets without blocking. Latency = completion
    seen by the sweep - scheduled arrival."""
    import threading
    import es_sieve
    reqs = workloads.serve_requests(n, seed=seed)
    tickets = [None] * n
    refused = [0]
    t0 = time.perf_counter() + 0.01

    def submitter():
        for i, (t, lo, hi) in enumerate(reqs):
            d = t0 + t - time.perf_counter()
            if d > 0:
                time.sleep(d)
            while True:
                try:
                    tickets[i] = eng.submit([(lo, hi)])
                    break
                except es_sieve.EsError as ex:
                    if ex.status != es_sieve.ES_ERR_BUSY:
                        raise
                    refused[0] += 1
                    time.sleep(0.0005)

    th = threading.Thread(target=submitter)
    th.start()
    done_at = [None] * n
    left = set(range(n))
    while left:
        for i in sorted(left):
            if tickets[i] is None:
                break
            try:
                eng.poll(tickets[i], 1, timeout_ms=0)
            except es_sieve.EsError as ex:
                if ex.status != es_sieve.ES_ERR_TIMEOUT:
                    raise
                continue
            done_at[i] = time.perf_counter()
            left.discard(i)
        time.sleep(0.00005)
    th.join()
    lat = [1000.0 * (done_at[i] - (t0 + reqs[i][0])) for i in range(n)]
    span = max(done_at) - (t0 + reqs[0][0])
    ints = sum(hi - lo for _, lo, hi in reqs)
    return {"requests": n, "arrivals": "poisson, mean gap 0.5 ms, lengths 2^12..2^30 log-uniform",
            "offered_integers_per_s": ints / reqs[-1][0], "integers_per_s": ints / span,
            "p50_ms": percentile(lat, 50), "p99_ms": percentile(lat, 99), "max_ms": max(lat),
            "busy_refusals": refused[0]}


def sync_leg(eng, wins, steps, flush):
    """`steps` synchronous es_run_batch calls from host buffers, L2 flushed before each: the
    device time of each call's kernels (es_timing, CUDA events on the engine's stream) and the
    wall time of the call."""
    out = {"dev_ms": 0.0, "wall_s": 0.0, "launches": 0, "recs": 0,
           "stage": {"mark_ms": 0.0, "mr_ms": 0.0, "rung_ms": 0.0, "direct_ms": 0.0},
           "kern": {"prep_ms": 0.0, "mark_short_ms": 0.0, "mark_long_ms": 0.0},
           "host": {"host_setup_ms": 0.0, "host_device_ms": 0.0, "host_collect_ms": 0.0, "host_total_ms": 0.0}}
    warr, carr = eng.make_windows(wins), eng.make_counters(len(wins))
    for _ in range(steps):
        flush()
        t0 = time.perf_counter()
        nrec = eng.run_batch_c(warr, len(wins), carr)     # es_run_batch: host buffers in and out
        out["wall_s"] += time.perf_counter() - t0
        t = eng.timing()
        out["last"] = t
        out["dev_ms"] += t["total_ms"]
        out["launches"] += int(t["kernel_launches"])
        out["recs"] = max(out["recs"], nrec)
        for grp in ("stage", "kern", "host"):
            for k in out[grp]:
                out[grp][k] += t[k]
    return out


def pipelined_leg(eng, wins, steps, warmup, flush_async, depth=3):
    """`steps` batches through es_submit_batch / es_poll from host buffers, `depth` of them
    submitted at a time: the engine's two serving streams each run one, marking one batch
    while the other's stage D finishes. A 256 MB L2-flushing write is queued before every
    submission (on another stream: it runs beside the batches in flight and competes with
    them). Returns (wall seconds of the timed steps, the largest record count of a step)."""
    from collections import deque
    n = len(wins)
    warr = eng.make_windows(wins)
    carrs = [eng.make_counters(n) for _ in range(depth)]

    def run(k):
        q, recs = deque(), 0
        t0 = time.perf_counter()
        for i in range(k):
            flush_async()
            q.append(eng.submit_batch_c(warr, n))
            if len(q) >= depth:
                recs = max(recs, eng.poll_c(q.popleft(), carrs[i % depth]))
        while q:
            recs = max(recs, eng.poll_c(q.popleft(), carrs[0]))
        return time.perf_counter() - t0, recs
    run(max(warmup, 2 * depth))
    return run(steps)


def roofline(args, wins, n_int, kern, stage, last_t, schedule, clocks):
    """The dominant kernel against the bound that binds it. k_mark_short is instruction-issue
    bound integer work: `achieved` is its warp instructions per launch (ncu, same schedule)
    over its live CUDA-event time, `peak` 152 SMs x 4 schedulers x one instruction per cycle at
    the sampled SM clock. Sub-objects: `hbm` (the kill-mask rows, stride residues and window
    list one launch reads, over the same time, against the measured copy bandwidth), `marks`
    (the per-mark view of a segment sieve) and `stage_d` (k_rung, latency-bound)."""
    hbm_peak, peak_kind = peaks()
    mhz = clocks.get("sm_mhz") or 2070.0
    peak_issue = 152 * 4 * mhz * 1e6
    per_kernel = {"k_mark_short": kern["mark_short_ms"], "k_mark": kern["mark_long_ms"], "k_prep": kern["prep_ms"],
                  "k_mr": stage["mr_ms"], "k_rung": stage["rung_ms"], "k_direct": stage["direct_ms"]}
    dom = max(per_kernel, key=per_kernel.get)
    ms = per_kernel[dom] / args.steps
    default = args.windows == 4096 and args.sieve == 0
    cap = MARK_SHORT_NCU.get((schedule["short_max"], schedule["long_split"])) if default else None
    if dom == "k_mark_short":
        # one kill-mask row per lane (as laid out: the interleaved rounds padded), the per-window
        # stride residues (u16 rows of 264) and the window list
        alg = last_t["mask_bytes"] + len(wins) * 264 * 2 + len(wins) * 32
    else:
        alg = int(last_t["primes"]) * (24 + 64)             # the survivor tail: 24 B in, 64 B out per prime
    roof = {"kernel": dom, "bound": "issue", "unit": "warp inst/s", "peak": peak_issue, "ms_per_launch": ms,
            "achieved": None, "frac": None, "traffic": cap["dram"] if cap and dom == "k_mark_short" else None,
            "schedule": schedule}
    if cap and dom == "k_mark_short":
        roof["achieved"] = cap["inst"] / (ms / 1000.0)
        roof["frac"] = roof["achieved"] / peak_issue
        roof["inst_per_launch"] = cap["inst"]
    else:
        roof["note"] = "no ncu capture for this kernel and schedule: no issue figure"
    gbs = alg / (ms / 1000.0) / 1e9
    roof["hbm"] = {"achieved": gbs, "peak": hbm_peak, "unit": "GB/s", "frac": gbs / hbm_peak, "peak_kind": peak_kind,
                   "algorithmic_bytes": alg, "traffic": roof["traffic"]}
    if dom == "k_mark_short" and args.sieve == 0:
        # The per-mark view: a segment sieve clears one bit per mark with a 4-byte shared-memory
        # read-modify-write (8 bytes); the kill-mask kernel does no per-mark work, so this is the
        # bandwidth such a sieve would need to match it, against the nominal shared-memory rate
        # (152 SMs x 128 B per cycle at the sampled clock).
        marks = n_int * MARKS_PER_INTEGER_GPU
        smem_peak = 152 * 128 * mhz * 1e6 / 1e9
        rmw_gbs = marks * 8 / (ms / 1000.0) / 1e9
        roof["marks"] = {"per_launch": marks, "achieved": marks / (ms / 1000.0), "unit": "marks/s",
                         "rmw_equivalent_gbs": rmw_gbs, "smem_peak_gbs": smem_peak, "peak_kind": "nominal",
                         "frac": rmw_gbs / smem_peak}
    rcap = RUNG_NCU.get(schedule["rung_blocks_per_sm"]) if default else None
    if stage["rung_ms"] > 0:
        # The survivor tail (stage D): integer-pipe work bound by the latency of its hardest
        # factorizations; the same issue arithmetic over k_rung's live time.
        rung_ms = stage["rung_ms"] / args.steps
        sd = {"kernel": "k_rung", "bound": "latency", "ms_per_launch": rung_ms, "issue": None}
        if rcap:
            rate = rcap["inst"] / (rung_ms / 1000.0)
            sd["issue"] = {"achieved": rate, "peak": peak_issue, "unit": "warp inst/s", "frac": rate / peak_issue,
                           "inst_per_launch": rcap["inst"]}
        roof["stage_d"] = sd
    return roof


def tuned_table_leg(args, rank, local, schedule, flush, flush_async):
    """Both batches with the GB300-tuned filter table instead of the reference's (same
    schedule): device time of the kernels (synchronous calls, L2 flushed) and the pipelined
    e2e, with the survivors and primes the table leaves."""
    import hashlib
    import es_sieve
    body = "".join(ln for ln in open(GB300_TABLE) if ln.startswith("FILTER "))
    out = {"table": os.path.basename(GB300_TABLE), "filters": body.count("\n"),
           "sha256": hashlib.sha256(body.encode()).hexdigest()}
    with es_sieve.Engine(wheel=2042040, filters=GB300_TABLE, device=local) as eng:
        eng.set_schedule(short_max=schedule["short_max"], rung_blocks_per_sm=schedule["rung_blocks_per_sm"],
                         long_split=schedule["long_split"])
        for name, wins in (("batch4096", workloads.batch_windows(args.windows, seed=workloads.SEED + rank)),
                           ("batch19", workloads.batch19_windows(args.windows, seed=workloads.SEED + rank))):
            n = integers(wins)
            for _ in range(args.warmup):
                eng.run_batch(wins, records=False)
            sy = sync_leg(eng, wins, args.steps, flush)
            pw, _ = pipelined_leg(eng, wins, args.steps, args.warmup, flush_async)
            out[name] = {"value": n * args.steps / (sy["dev_ms"] / 1000.0), "ms_per_step": sy["dev_ms"] / args.steps,
                         "stages_ms_per_step": dict({k: v / args.steps for k, v in sy["stage"].items()},
                                                    **{k: v / args.steps for k, v in sy["kern"].items()}),
                         "survivors": int(sy["last"]["survivors"]), "primes": int(sy["last"]["primes"]),
                         "e2e": {"value": n * args.steps / pw, "ms_per_step": 1000.0 * pw / args.steps,
                                 "mode": "pipelined (es_submit_batch / es_poll, 3 in flight)"}}
    return out


def run_gpu(args, ws, rank, local):
    import es_sieve
    flush, flush_async, flush_note = l2_flusher(local)
    mods, ress = es_sieve.load_filters(GPU_TABLE)
    eng = es_sieve.Engine(wheel=2042040, filters=(mods, ress), device=local, sieve_p=args.sieve)
    wins = workloads.batch_windows(args.windows, seed=workloads.SEED + rank)
    n_int = integers(wins)
    if args.schedule:
        sm, rb, ls = (int(x) for x in args.schedule.split(","))
        eng.set_schedule(short_max=sm, rung_blocks_per_sm=rb, long_split=ls)
        schedule = eng.schedule()
    else:
        schedule = eng.autotune(wins, repeats=6) if not args.no_autotune else eng.schedule()
    for _ in range(args.warmup):
        eng.run_batch(wins)
    barrier(ws)
    with Clocks(local) as clk:
        sy = sync_leg(eng, wins, args.steps, flush)
        if args.no_pipelined:
            pipe_wall, pipe_recs = sy["wall_s"], sy["recs"]
        else:
            pipe_wall, pipe_recs = pipelined_leg(eng, wins, args.steps, args.warmup, flush_async)
    barrier(ws)
    clocks = clk.summary()
    dev_ms, wall_s, launches, recs_n = sy["dev_ms"], sy["wall_s"], sy["launches"], sy["recs"]
    stage, kern, host, last_t = sy["stage"], sy["kern"], sy["host"], sy["last"]
    dev_s = allmax(ws, dev_ms / 1000.0)
    wall = allmax(ws, wall_s)
    pipe = allmax(ws, pipe_wall)
    total_int = allsum(ws, n_int * args.steps)
    value = total_int / dev_s
    e2e_sync = total_int / wall
    e2e = total_int / pipe
    extra = {}
    if not args.no_plain:
        flush()
        per_p, rec_p = eng.run_batch(wins, schedule=es_sieve.ES_SCHED_PLAIN)
        tp = eng.timing()
        extra["plain"] = {"value": n_int / (tp["total_ms"] / 1000.0), "ms_per_step": tp["total_ms"],
                          "kernel_launches": int(tp["kernel_launches"])}
        per_b, rec_b = eng.run_batch(wins)
        extra["plain"]["counters_identical"] = per_p == per_b
        extra["plain"]["records_identical"] = rec_p.tobytes() == rec_b.tobytes()
        c3 = workloads.c3()
        eng.run_window(c3["lo"], c3["hi"])
        flush()
        eng.run_window(c3["lo"], c3["hi"])
        t3 = eng.timing()
        extra["c3"] = {"value": (c3["hi"] - c3["lo"]) / (t3["total_ms"] / 1000.0), "ms_per_step": t3["total_ms"],
                       "lo": c3["lo"], "mark_ms": t3["mark_ms"], "rung_ms": t3["rung_ms"]}
    if not args.no_batch19:
        # the same batch law at the top of the range, [1e19, DIRECT_PMAX): same engine and schedule
        w19 = workloads.batch19_windows(args.windows, seed=workloads.SEED + rank)
        n19 = integers(w19)
        for _ in range(args.warmup):
            eng.run_batch(w19)
        s19 = sync_leg(eng, w19, args.steps, flush)
        p19, _ = pipelined_leg(eng, w19, args.steps, args.warmup, flush_async)
        b19 = {"windows": len(w19), "integers_per_step": n19,
               "value": n19 * args.steps / (s19["dev_ms"] / 1000.0), "ms_per_step": s19["dev_ms"] / args.steps,
               "stages_ms_per_step": dict({k: v / args.steps for k, v in s19["stage"].items()},
                                          **{k: v / args.steps for k, v in s19["kern"].items()}),
               "primes": int(s19["last"]["primes"]),
               "e2e": {"value": n19 * args.steps / p19, "mode": "pipelined (es_submit_batch / es_poll, 3 in flight)"},
               "e2e_sync": {"value": n19 * args.steps / s19["wall_s"], "mode": "es_run_batch"}}
        if not args.no_plain:
            flush()
            eng.run_batch(w19, schedule=es_sieve.ES_SCHED_PLAIN, records=False)
            tp = eng.timing()
            b19["plain"] = {"value": n19 / (tp["total_ms"] / 1000.0), "ms_per_step": tp["total_ms"],
                            "kernel_launches": int(tp["kernel_launches"])}
        extra["batch19"] = b19
    if not args.no_tuned_table and args.sieve == 0:
        extra["gb300_table"] = tuned_table_leg(args, rank, local, schedule, flush, flush_async)
    if args.serve:
        serve_leg(eng, min(200, args.serve), workloads.SEED + 7)          # warm the serving slots
        extra["serve"] = serve_leg(eng, args.serve, workloads.SEED + 1000 * (rank + 1))
    roof = roofline(args, wins, n_int, kern, stage, last_t, schedule, clocks)
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        # the same fixed sample through both: the oracle port on every host thread, and the
        # engine (device time of a synchronous es_run_batch, and its wall time from host buffers)
        sample = wins[:args.cpu_windows]
        rate, done, cores, el = cpu_baseline(sample, float("inf"))
        for _ in range(2):
            eng.run_batch(sample, records=False)
        flush()
        t0 = time.perf_counter()
        eng.run_batch(sample)
        wall_sample = time.perf_counter() - t0
        ts = eng.timing()
        cpu = {"value": rate, "unit": "integers/s", "cores": cores, "kind": "port",
               "sample": "the first %d windows of the batch (%d integers, %.1f s, all host threads)"
                         % (done, integers(sample), el), "host": host_cpu(),
               "gpu_on_sample": {"value": integers(sample) / (ts["total_ms"] / 1000.0),
                                 "e2e": integers(sample) / wall_sample, "mode": "es_run_batch"}}
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "integers/s", "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1000.0 * dev_s / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "u64", "data": "synthetic",
                "config": {"workload": "batch4096", "windows": args.windows, "integers_per_step": n_int,
                           "wheel": 2042040, "filters": "f_M2042040_mmax2000_gpu.txt", "seed": workloads.SEED,
                           "sieve": args.sieve,
                           "schedule": "persistent", "kernel_schedule": schedule, "l2": flush_note,
                           "parallelism": "replicas x%d" % ws},
                # copied every step: batch header, window and short-window descriptors in; run
                # counters, status, per-window counters and records out (pinned staging; the
                # graph copies the first 4096 record slots back every run, any more afterwards)
                "e2e": {"value": e2e, "unit": "integers/s", "h2d_bytes_per_step": 16 + len(wins) * (48 + 32),
                        "d2h_bytes_per_step": 68 + 64 * len(wins) + 64 * max(pipe_recs, 4096),
                        "mode": ("es_run_batch, one call per step" if args.no_pipelined else
                                 "pipelined: es_submit_batch / es_poll, 3 batches in flight, host buffers in and out"),
                        "ms_per_step": 1000.0 * pipe / args.steps},
                "e2e_sync": {"value": e2e_sync, "unit": "integers/s", "mode": "es_run_batch, one call per step",
                             "h2d_bytes_per_step": 16 + len(wins) * (48 + 32),
                             "d2h_bytes_per_step": 68 + 64 * len(wins) + 64 * max(recs_n, 4096),
                             "ms_per_step": 1000.0 * wall / args.steps},
                "gpu_launches": launches + (0 if args.no_pipelined else int(last_t["kernel_launches"]) * args.steps),
                "clocks": clocks,
                "roofline": roof, "cpu_baseline": cpu,
                "stages_ms_per_step": dict({k: v / args.steps for k, v in stage.items()},
                                           **{k: v / args.steps for k, v in kern.items()}),
                "tail": {"survivors": int(last_t["survivors"]), "primes": int(last_t["primes"])},
                # where the e2e call's wall time goes (es_timing host fields), per step
                "e2e_host_ms_per_step": {k[5:]: v / args.steps for k, v in host.items()}}
        line.update(extra)
        print(json.dumps(line))
    eng.close()


def main():
    args = parse()
    ws, rank, local = dist()
    if args.impl == "reference":
        run_reference(args, ws, rank)
    else:
        run_gpu(args, ws, rank, local)
    if ws > 1:
        import torch.distributed as td
        td.destroy_process_group()


if __name__ == "__main__":
    main()
