"""Python binding of the GB300 verification-sieve engine (ctypes over include/es_sieve.h).

The reference's surface for this path is rung_scan3's command line and its sweep seam
(sieve/rung_scan3.cpp:711-784, :960-1163). This module mirrors it for Python callers:

    eng = Engine(wheel=2042040, filters="f_M2042040_mmax2000_gpu.txt")
    counters, records = eng.run_window(lo, hi)          # lane-major records, SUMMARY counters
    text = eng.stream(lo, hi)                           # byte-identical to rung_scan3's stdout
    per_window, records = eng.run_batch(windows)        # many windows, one persistent launch

There is no fallback: if libes_sieve.so is missing or no GPU is present, the calls raise.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libes_sieve.so")
CLI_PATH = os.path.join(HERE, "rung_scan3_gb300")

ES_OK, ES_ERR_ARG, ES_ERR_PIN, ES_ERR_RANGE, ES_ERR_FILTERS, ES_ERR_CUDA, ES_ERR_DEVICE_STATUS, \
    ES_ERR_NOMEM, ES_ERR_TIMEOUT, ES_ERR_BUSY = range(10)
ES_REC_RUNG, ES_REC_SOLVED, ES_REC_SURVIVOR = 1, 2, 3
ES_SCHED_PLAIN, ES_SCHED_PERSISTENT = 0, 1

COUNTER_NAMES = ("positions", "covered", "sieved", "mr", "composite", "rung", "direct", "survivors")


class EsError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (status, msg))
        self.status = status


class Config(C.Structure):
    _fields_ = [("wheel_M", C.c_uint64), ("mmax", C.c_uint64), ("sieve_p", C.c_uint64), ("seg", C.c_uint64),
                ("filter_mods", C.POINTER(C.c_uint64)), ("filter_ress", C.POINTER(C.c_uint64)),
                ("n_filters", C.c_size_t), ("device", C.c_int), ("mem_budget", C.c_size_t), ("flags", C.c_uint32)]


class Counters(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in COUNTER_NAMES]

    def as_dict(self):
        return {n: int(getattr(self, n)) for n in COUNTER_NAMES}


RECORD_DTYPE = np.dtype([("kind", "<u4"), ("window", "<u4"), ("lane", "<u4"), ("reserved", "<u4"),
                         ("J", "<u8"), ("p", "<u8"), ("a", "<u8"), ("b", "<u8"), ("c", "<u8"), ("d", "<u8")])


class Record(C.Structure):
    _fields_ = [(n, C.c_uint32) for n in ("kind", "window", "lane", "reserved")] + \
               [(n, C.c_uint64) for n in ("J", "p", "a", "b", "c", "d")]


class Records(C.Structure):
    _fields_ = [("recs", C.POINTER(Record)), ("n", C.c_size_t)]


class Window(C.Structure):
    _fields_ = [("lo", C.c_uint64), ("hi", C.c_uint64)]


class Info(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in ("wheel_M", "lanes", "wheel_pmin", "cover_pmax", "floor", "ceiling",
                                          "class_fnv64", "filter_fnv64", "n_certified", "n_filters", "mmax",
                                          "short_max_limit")] + \
               [("pinned", C.c_int), ("classes_sha256", C.c_char * 72)]


class Schedule(C.Structure):
    _fields_ = [("short_max", C.c_uint32), ("rung_blocks_per_sm", C.c_uint32), ("long_split", C.c_uint32),
                ("reserved", C.c_uint32 * 5)]

    def as_dict(self):
        return {"short_max": int(self.short_max), "rung_blocks_per_sm": int(self.rung_blocks_per_sm),
                "long_split": int(self.long_split)}


class Timing(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("total_ms", "mark_ms", "mr_ms", "rung_ms", "direct_ms", "prep_ms",
                                          "mark_short_ms", "mark_long_ms")] + \
               [(n, C.c_uint64) for n in ("marks_kernel_launches", "kernel_launches", "mark_items", "survivors",
                                          "primes", "short_pairs", "mask_bytes")] + \
               [(n, C.c_double) for n in ("host_setup_ms", "host_device_ms", "host_collect_ms", "host_total_ms")]


_lib = None


def load_library(path=LIB_PATH):
    """Load libes_sieve.so and declare its signatures. Raises if the library is absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise FileNotFoundError("libes_sieve.so not built (run __graft_entry__.build()): " + path)
    lib = C.CDLL(path)
    P = C.POINTER
    e = C.c_void_p
    sig = {
        "es_open": (C.c_int, [P(Config), P(C.c_void_p)]),
        "es_close": (C.c_int, [e]),
        "es_load_filters": (C.c_int, [C.c_char_p, P(P(C.c_uint64)), P(P(C.c_uint64)), P(C.c_size_t)]),
        "es_free_u64": (None, [P(C.c_uint64)]),
        "es_run_window": (C.c_int, [e, C.c_uint64, C.c_uint64, P(Counters), P(Records)]),
        "es_run_batch": (C.c_int, [e, P(Window), C.c_size_t, C.c_int, P(Counters), P(Records)]),
        "es_submit": (C.c_int, [e, P(Window), C.c_size_t, P(C.c_uint64)]),
        "es_submit_batch": (C.c_int, [e, P(Window), C.c_size_t, P(C.c_uint64)]),
        "es_poll": (C.c_int, [e, C.c_uint64, P(Counters), P(Records), C.c_int]),
        "es_free_records": (C.c_int, [P(Records)]),
        "es_format_record": (C.c_size_t, [P(Record), C.c_char_p, C.c_size_t]),
        "es_format_summary": (C.c_size_t, [e, C.c_uint64, C.c_uint64, P(Counters), C.c_char_p, C.c_size_t]),
        "es_info": (C.c_int, [e, P(Info)]),
        "es_get_schedule": (C.c_int, [e, P(Schedule)]),
        "es_set_schedule": (C.c_int, [e, P(Schedule)]),
        "es_autotune": (C.c_int, [e, P(Window), C.c_size_t, C.c_int, P(Schedule)]),
        "es_classes": (C.c_int, [e, P(C.c_uint64), C.c_size_t]),
        "es_timing": (C.c_int, [e, P(Timing)]),
        "es_status_str": (C.c_char_p, [C.c_int]),
        "es_last_error": (C.c_char_p, [e]),
        "es_is_prime_batch": (C.c_int, [e, P(C.c_uint64), C.c_size_t, P(C.c_uint8)]),
        "es_solve_rung_batch": (C.c_int, [e, P(C.c_uint64), C.c_size_t, P(Record), P(C.c_uint8)]),
        "es_solve_direct_batch": (C.c_int, [e, P(C.c_uint64), C.c_size_t, P(Record), P(C.c_uint8)]),
        "es_factor_batch": (C.c_int, [e, P(C.c_uint64), C.c_size_t, P(C.c_uint64), P(C.c_uint8), P(C.c_uint8)]),
        "es_check_records": (C.c_int, [e, P(Record), C.c_size_t, P(C.c_uint8)]),
        "es_sha256_hex": (C.c_size_t, [C.c_void_p, C.c_size_t, C.c_char_p, C.c_size_t]),
        "es_is_prime_noalloc": (C.c_int, [C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def load_filters(path):
    """FILTER lines of a filter table as two uint64 arrays (sieve/rung_scan3.cpp:1080-1097)."""
    mods, ress = [], []
    with open(path) as f:
        for line in f:
            t = line.split()
            if len(t) >= 3 and t[0] == "FILTER":
                mods.append(int(t[1]))
                ress.append(int(t[2]))
    return np.array(mods, dtype=np.uint64), np.array(ress, dtype=np.uint64)


def _u64p(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint64))


def format_record(rec):
    """Text line of one record row (numpy structured row or Record)."""
    lib = load_library()
    r = Record(*[int(rec[n]) for n in RECORD_DTYPE.names])
    buf = C.create_string_buffer(200)
    n = lib.es_format_record(C.byref(r), buf, 200)
    return buf.raw[:n].decode()


class Engine:
    def __init__(self, wheel=2042040, mmax=10000, sieve_p=0, filters=None, device=0, no_rung=False, mem_budget=0,
                 test_rho_budget=False):
        """filters: None (the generated default set), a filter-file path, or (mods, ress)."""
        self.lib = load_library()
        if isinstance(filters, str):
            filters = load_filters(filters)
        cfg = Config()
        cfg.wheel_M, cfg.mmax, cfg.sieve_p, cfg.device = wheel, mmax, sieve_p, device
        cfg.flags = (1 if no_rung else 0) | (2 if test_rho_budget else 0)
        cfg.mem_budget = mem_budget
        self._keep = None
        if filters is not None:
            mods = np.ascontiguousarray(filters[0], dtype=np.uint64)
            ress = np.ascontiguousarray(filters[1], dtype=np.uint64)
            self._keep = (mods, ress)
            cfg.filter_mods, cfg.filter_ress, cfg.n_filters = _u64p(mods), _u64p(ress), len(mods)
        h = C.c_void_p()
        st = self.lib.es_open(C.byref(cfg), C.byref(h))
        if st != ES_OK:
            raise EsError(st, (self.lib.es_last_error(None) or b"").decode())
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.es_close(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, st):
        if st != ES_OK:
            raise EsError(st, (self.lib.es_last_error(self.h) or b"").decode())

    def info(self):
        i = Info()
        self._check(self.lib.es_info(self.h, C.byref(i)))
        d = {n: int(getattr(i, n)) for n, _ in Info._fields_ if n not in ("classes_sha256", "pinned")}
        d["pinned"] = bool(i.pinned)
        d["classes_sha256"] = i.classes_sha256.decode()
        return d

    def classes(self):
        n = self.info()["lanes"]
        out = np.zeros(n, dtype=np.uint64)
        self._check(self.lib.es_classes(self.h, _u64p(out), n))
        return out

    def timing(self):
        t = Timing()
        self._check(self.lib.es_timing(self.h, C.byref(t)))
        return {n: getattr(t, n) for n, _ in Timing._fields_}

    @staticmethod
    def _take_records(lib, recs):
        n = recs.n
        if n:
            buf = (C.c_char * (n * RECORD_DTYPE.itemsize)).from_address(C.addressof(recs.recs.contents))
            arr = np.frombuffer(bytes(buf), dtype=RECORD_DTYPE).copy()
        else:
            arr = np.zeros(0, dtype=RECORD_DTYPE)
        lib.es_free_records(C.byref(recs))
        return arr

    def run_window(self, lo, hi, records=True):
        c = Counters()
        r = Records()
        self._check(self.lib.es_run_window(self.h, lo, hi, C.byref(c), C.byref(r) if records else None))
        return c.as_dict(), (self._take_records(self.lib, r) if records else None)

    def run_batch(self, windows, schedule=ES_SCHED_PERSISTENT, records=True):
        n = len(windows)
        w = self.make_windows(windows)
        c = (Counters * max(n, 1))()
        r = Records()
        self._check(self.lib.es_run_batch(self.h, w, n, schedule, c, C.byref(r) if records else None))
        return [c[i].as_dict() for i in range(n)], (self._take_records(self.lib, r) if records else None)

    # The C call alone, for timing: caller-built window and counter arrays (make_windows,
    # make_counters), records freed here; returns the record count.
    @staticmethod
    def make_windows(windows):
        """A ctypes es_window array from (lo, hi) pairs, built through numpy (no per-window
        Python objects)."""
        a = np.zeros((max(len(windows), 1), 2), dtype=np.uint64)
        if len(windows):
            a[:len(windows)] = np.asarray(windows, dtype=np.uint64).reshape(-1, 2)
        return (Window * len(a)).from_buffer_copy(a.tobytes())

    @staticmethod
    def make_counters(n):
        return (Counters * max(n, 1))()

    def run_batch_c(self, warr, n, carr, schedule=ES_SCHED_PERSISTENT):
        r = Records()
        self._check(self.lib.es_run_batch(self.h, warr, n, schedule, carr, C.byref(r)))
        nrec = r.n
        self.lib.es_free_records(C.byref(r))
        return nrec

    # ------------------------------------------------------------------ schedule
    def schedule(self):
        sc = Schedule()
        self._check(self.lib.es_get_schedule(self.h, C.byref(sc)))
        return sc.as_dict()

    def set_schedule(self, short_max=None, rung_blocks_per_sm=None, long_split=None):
        sc = Schedule()
        self._check(self.lib.es_get_schedule(self.h, C.byref(sc)))
        if short_max is not None:
            sc.short_max = short_max
        if rung_blocks_per_sm is not None:
            sc.rung_blocks_per_sm = rung_blocks_per_sm
        if long_split is not None:
            sc.long_split = long_split
        self._check(self.lib.es_set_schedule(self.h, C.byref(sc)))

    def autotune(self, windows, repeats=6):
        """Time the candidate schedules on these windows (`repeats` timed runs each), keep the
        one with the lowest mean device time; returns it."""
        n = len(windows)
        w = self.make_windows(windows)
        sc = Schedule()
        self._check(self.lib.es_autotune(self.h, w, n, repeats, C.byref(sc)))
        return sc.as_dict()

    # ------------------------------------------------------------------ serving
    def submit(self, windows):
        """Queue windows; returns a ticket. Raises EsError(ES_ERR_BUSY) when admission is refused."""
        n = len(windows)
        w = self.make_windows(windows)
        t = C.c_uint64()
        self._check(self.lib.es_submit(self.h, w, n, C.byref(t)))
        return t.value

    def submit_batch(self, windows):
        """Queue windows as one batch of their own (es_submit_batch); returns a ticket for poll()."""
        n = len(windows)
        w = self.make_windows(windows)
        return self.submit_batch_c(w, n)

    # The C calls alone, for timing: a caller-built window array (make_windows) in, a
    # caller-built counter array (make_counters) filled, records freed here.
    def submit_batch_c(self, warr, n):
        t = C.c_uint64()
        self._check(self.lib.es_submit_batch(self.h, warr, n, C.byref(t)))
        return t.value

    def poll_c(self, ticket, carr, timeout_ms=-1):
        """es_poll into carr; returns the record count."""
        r = Records()
        self._check(self.lib.es_poll(self.h, ticket, carr, C.byref(r), timeout_ms))
        nrec = r.n
        self.lib.es_free_records(C.byref(r))
        return nrec

    def poll(self, ticket, n, timeout_ms=-1):
        """(per-window counters, records) of a submitted request; EsError(ES_ERR_TIMEOUT) if not done."""
        c = (Counters * max(n, 1))()
        r = Records()
        self._check(self.lib.es_poll(self.h, ticket, c, C.byref(r), timeout_ms))
        return [c[i].as_dict() for i in range(n)], self._take_records(self.lib, r)

    def summary(self, lo, hi, counters):
        c = Counters(*[counters[n] for n in COUNTER_NAMES])
        buf = C.create_string_buffer(600)
        n = self.lib.es_format_summary(self.h, lo, hi, C.byref(c), buf, 600)
        return buf.raw[:n].decode()

    def text(self, lo, hi, counters, records, emit_survivors=True):
        """The reference's stdout record for one window: lines in lane order, then SUMMARY."""
        lines = [format_record(r) for r in records if emit_survivors or r["kind"] != ES_REC_SURVIVOR]
        return "".join(lines) + self.summary(lo, hi, counters)

    def stream(self, lo, hi, emit_survivors=True):
        c, r = self.run_window(lo, hi)
        return self.text(lo, hi, c, r, emit_survivors)

    # ------------------------------------------------------------------ probes
    def is_prime(self, ns):
        a = np.ascontiguousarray(ns, dtype=np.uint64)
        out = np.zeros(len(a), dtype=np.uint8)
        self._check(self.lib.es_is_prime_batch(self.h, _u64p(a), len(a), out.ctypes.data_as(C.POINTER(C.c_uint8))))
        return out.astype(bool)

    def _solve(self, fn, ps):
        a = np.ascontiguousarray(ps, dtype=np.uint64)
        recs = (Record * max(len(a), 1))()
        found = np.zeros(len(a), dtype=np.uint8)
        self._check(fn(self.h, _u64p(a), len(a), recs, found.ctypes.data_as(C.POINTER(C.c_uint8))))
        out = []
        for i in range(len(a)):
            out.append(format_record({n: getattr(recs[i], n) for n in RECORD_DTYPE.names}) if found[i] else None)
        return out

    def solve_rung(self, ps):
        """Certificate line per prime (solve_rung3), or None."""
        return self._solve(self.lib.es_solve_rung_batch, ps)

    def solve_direct(self, ps):
        """Certificate line per prime (solve_direct3), or None."""
        return self._solve(self.lib.es_solve_direct_batch, ps)

    def check_records(self, recs):
        """Device re-check of certificate records (a RECORD_DTYPE array): a bool array."""
        a = np.ascontiguousarray(recs, dtype=RECORD_DTYPE)
        out = np.zeros(len(a), dtype=np.uint8)
        self._check(self.lib.es_check_records(self.h, a.ctypes.data_as(C.POINTER(Record)), len(a),
                                              out.ctypes.data_as(C.POINTER(C.c_uint8))))
        return out.astype(bool)

    def factor(self, ns):
        a = np.ascontiguousarray(ns, dtype=np.uint64)
        pr = np.zeros(len(a) * 16, dtype=np.uint64)
        ex = np.zeros(len(a) * 16, dtype=np.uint8)
        k = np.zeros(len(a), dtype=np.uint8)
        u8 = C.POINTER(C.c_uint8)
        self._check(self.lib.es_factor_batch(self.h, _u64p(a), len(a), _u64p(pr), ex.ctypes.data_as(u8),
                                             k.ctypes.data_as(u8)))
        return [[(int(pr[i * 16 + j]), int(ex[i * 16 + j])) for j in range(k[i])] for i in range(len(a))]
