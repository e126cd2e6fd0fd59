/* es_sieve.h -- C ABI of the GB300 engine for the Erdos-Straus verification sieve's
 * per-window funnel: wheel filtering against the certified class table, marking of the
 * self-certifying cover progressions (and optional stage-B' small primes), survivor
 * compaction, deterministic 64-bit Miller-Rabin, the rung walk (stage D) and the direct
 * search (stage E) -- all on one GPU, results identical to the reference scanner.
 *
 * The reference exposes this path as a command line (sieve/rung_scan3.cpp:960-1163)
 * over an in-process seam: sweep_lane (:711-784), solve_rung3 (:578), solve_direct3
 * (:624). Each entry point below names the piece of that surface it replaces.
 *
 * Conventions: plain C types, caller-owned inputs, engine-allocated record arrays that the
 * caller frees with es_free_records. Every failure is a status code; nothing aborts.
 * One engine owns one GPU stream; use one engine per host thread (es_submit/es_poll are
 * the exception: they are safe to call from several threads on one engine).
 */
#ifndef ES_SIEVE_H
#define ES_SIEVE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. The reference's CLI exits 1 on every refusal (sieve/rung_scan3.cpp:
 * 1009-1015 unknown flag, :1041-1048 pin drift, :1057-1069 ceiling/floor, :1086/:1095
 * filter file); here each refusal has its own code. */
typedef enum {
  ES_OK = 0,
  ES_ERR_ARG = 1,           /* invalid argument or unsupported parameter */
  ES_ERR_PIN = 2,           /* derived class table does not match its pinned digest */
  ES_ERR_RANGE = 3,         /* LO <= the filter table's pmin floor, or HI > the stage-E ceiling */
  ES_ERR_FILTERS = 4,       /* filter file unreadable or holding no FILTER line */
  ES_ERR_CUDA = 5,          /* CUDA runtime failure: no device, launch or copy error */
  ES_ERR_DEVICE_STATUS = 6, /* a bounded device loop gave up (see es_last_error) */
  ES_ERR_NOMEM = 7,         /* device or host allocation failed */
  ES_ERR_TIMEOUT = 8,       /* es_poll: the ticket did not finish within timeout_ms */
  ES_ERR_BUSY = 9           /* es_submit: admission refused (no free slot or memory) */
} es_status;

/* Engine configuration (the flags of sieve/rung_scan3.cpp:984-1016). */
typedef struct {
  uint64_t wheel_M;             /* --wheel; 0 means 2042040 */
  uint64_t mmax;                /* --mmax; 0 means 10000 (default filter set and pmin floor) */
  uint64_t sieve_p;             /* --sieve: stage-B' primes <= sieve_p not dividing M; 0 = off */
  uint64_t seg;                 /* --seg: accepted for command-line parity; the device picks its
                                   own segment (results do not depend on it); 0 = default */
  const uint64_t *filter_mods;  /* --filters: certified (mod,res) pairs in file order; NULL =
                                   the generated default set (covers with m <= mmax, m not | M) */
  const uint64_t *filter_ress;
  size_t n_filters;
  int device;                   /* CUDA device ordinal */
  size_t mem_budget;            /* device bytes the engine may hold for work buffers; 0 = auto */
  uint32_t flags;               /* ES_FLAG_* */
} es_config;

/* Test hook of the frozen reference sieve (cover_scan --no-rung, sieve/cover_scan.cpp:395,
 * :431): skip stage D so that every prime goes to the direct search. */
#define ES_FLAG_NO_RUNG 1u
/* Test hook for the device-failure path: Brent's rho gives up after 64 steps per lane instead
 * of 2^24, so a cofactor with two large prime factors exhausts it; the run then fails with
 * ES_ERR_DEVICE_STATUS ("rho-budget") instead of emitting anything, and the engine stays
 * usable. Never set in production. */
#define ES_FLAG_TEST_RHO_BUDGET 2u

/* SUMMARY counters (Scan3Stats, sieve/rung_scan3.cpp:651-660). */
typedef struct {
  uint64_t positions, covered, sieved, mr, composite, rung, direct, survivors;
} es_counters;

/* One certificate or survivor, binary. es_format_record renders it as the reference's
 * text line (sieve/rung_scan3.cpp:595-599, :639-641, :781). */
enum { ES_REC_RUNG = 1, ES_REC_SOLVED = 2, ES_REC_SURVIVOR = 3 };
typedef struct {
  uint32_t kind;     /* ES_REC_* */
  uint32_t window;   /* index of the window within its batch (0 for es_run_window) */
  uint32_t lane;     /* lane index in wheel order */
  uint32_t reserved;
  uint64_t J;        /* position index within the lane, from the lane's first position */
  uint64_t p;        /* the prime */
  uint64_t a;        /* RUNG: A = (p+r)/4     SOLVED: a */
  uint64_t b;        /* RUNG: r               SOLVED: c */
  uint64_t c;        /* RUNG: u, low 64 bits  SOLVED: d */
  uint64_t d;        /* RUNG: u, high 64 bits SOLVED: k */
} es_record;

/* Records of a run, sorted by (window, lane, J): per window exactly the reference's
 * lane-major emission order (sieve/rung_scan3.cpp:1146-1151). */
typedef struct {
  es_record *recs;
  size_t n;
} es_records;

typedef struct { uint64_t lo, hi; } es_window;

/* Opaque engine handle. */
typedef struct es_engine es_engine;

/* What the engine derived at es_open (the stderr banner, sieve/rung_scan3.cpp:1120-1126,
 * and the SUMMARY's fixed fields, :1153-1158). */
typedef struct {
  uint64_t wheel_M;
  uint64_t lanes;
  uint64_t wheel_pmin;      /* max pmin over covers with m | M */
  uint64_t cover_pmax;      /* max pmin over all covers with m <= mmax */
  uint64_t floor;           /* LO must exceed this */
  uint64_t ceiling;         /* HI must not exceed this (DIRECT_PMAX) */
  uint64_t class_fnv64;
  uint64_t filter_fnv64;    /* FNV-1a over "mod,res;" of the certified filters */
  uint64_t n_certified;     /* ncov */
  uint64_t n_filters;       /* certified + stage-B' primes */
  uint64_t mmax;
  uint64_t short_max_limit; /* largest es_schedule.short_max (the kill-mask repeat, positions) */
  int pinned;               /* 1 if M has a pinned class-table digest */
  char classes_sha256[72];  /* the pin, or "unpinned" */
} es_info_t;

/* Device time of the last run, per stage, from CUDA events on the engine's stream;
 * total_ms is the sum of the stages (kernels only: no host<->device copies). */
typedef struct {
  double total_ms, mark_ms, mr_ms, rung_ms, direct_ms;
  double prep_ms, mark_short_ms, mark_long_ms;   /* the three parts of mark_ms */
  uint64_t marks_kernel_launches, kernel_launches;
  uint64_t mark_items, survivors, primes;
  uint64_t short_pairs;     /* (lane, short window) pairs, active or not, walked by k_mark_short */
  uint64_t mask_bytes;      /* kill-mask table bytes one k_mark_short launch reads */
  /* host wall time of the call: describing and staging the windows, from the launch to the
   * end of the device work (copies included), and collecting counters and records; and the
   * whole es_run_batch / es_run_window call inside the library (with the long-window split,
   * the three above are summed over its passes and host_total_ms also holds the split's own
   * work) */
  double host_setup_ms, host_device_ms, host_collect_ms, host_total_ms;
} es_timing_t;

/* Batch schedules: per-window launches of the same kernels, or one persistent launch over
 * a device work queue replayed from a CUDA graph. */
enum { ES_SCHED_PLAIN = 0, ES_SCHED_PERSISTENT = 1 };

/* Derive and pin the wheel, load the filters, build the device tables. Replaces the
 * setup of sieve/rung_scan3.cpp:1029-1126 (gen_covers, gen_wheel_covers, gen_ucerts,
 * build_wheel, the pin check, filter loading and stage-B' append). */
es_status es_open(const es_config *cfg, es_engine **engine_out);
es_status es_close(es_engine *engine);

/* Read a filter file ("FILTER mod res ..." lines, anything else ignored) into malloc'ed
 * arrays, as sieve/rung_scan3.cpp:1080-1097 does. Free with es_free_u64. */
es_status es_load_filters(const char *path, uint64_t **mods, uint64_t **ress, size_t *n);
void es_free_u64(uint64_t *p);

/* Verify every prime in [lo, hi): replaces the lane loop and merge of
 * sieve/rung_scan3.cpp:1132-1151 over sweep_lane (:711-784). Refuses floors and
 * ceilings like :1057-1069. recs may be NULL (counters only). */
es_status es_run_window(es_engine *engine, uint64_t lo, uint64_t hi, es_counters *out, es_records *recs);

/* Many windows at once: per_window[i] gets window i's counters; records carry their
 * window index. schedule is ES_SCHED_PLAIN or ES_SCHED_PERSISTENT. No reference
 * counterpart: the reference runs one window per process. */
es_status es_run_batch(es_engine *engine, const es_window *w, size_t n, int schedule,
                       es_counters *per_window, es_records *recs);

/* Serving: queue windows for verification without waiting; collect them by ticket.
 * Requests are batched continuously: whenever one of the engine's serving streams frees up,
 * it takes every queued request that fits its next batch, so requests that arrive while
 * others run join the next batch and batches on different streams overlap on the device.
 * Admission: ES_ERR_BUSY when the queue is full or the request's device-memory estimate does
 * not fit the engine's budget (es_config.mem_budget; 0 = a quarter of the free memory at
 * es_open); ES_ERR_RANGE at once for a window the run would refuse. es_poll waits up to
 * timeout_ms (negative: without limit; 0: just checks) and returns ES_ERR_TIMEOUT if the
 * request is not done; otherwise it fills per_window (one entry per submitted window) and
 * recs (window indices relative to the request) and forgets the ticket. A ticket has one
 * poller at a time: a second es_poll on a ticket that is being waited on returns ES_ERR_ARG.
 * es_close waits for es_poll calls already inside the engine; no call may start on an engine
 * after es_close has begun. No reference counterpart. */
es_status es_submit(es_engine *engine, const es_window *w, size_t n, uint64_t *ticket);
es_status es_poll(es_engine *engine, uint64_t ticket, es_counters *per_window, es_records *recs,
                  int timeout_ms);
/* The asynchronous form of es_run_batch (persistent schedule): the windows are queued as one
 * batch of their own (never merged with other requests, any number of windows) and collected
 * with es_poll like any ticket. Batches are marked one at a time in the order the serving
 * streams launch them, and each batch's stage D (a few latency-bound factorizations at the end
 * of its run) overlaps the next batch's marking, so a caller that keeps two batches submitted
 * verifies more integers/s than one calling es_run_batch in a loop. Admission as es_submit.
 * No reference counterpart. */
es_status es_submit_batch(es_engine *engine, const es_window *w, size_t n, uint64_t *ticket);

es_status es_free_records(es_records *recs);

/* One record as its text line, newline included; returns the length (0 if cap is too
 * small). The formats of sieve/rung_scan3.cpp:595-599, :639-641 and :781. */
size_t es_format_record(const es_record *r, char *buf, size_t cap);

/* The SUMMARY line (newline included) for a window's counters, exactly as
 * sieve/rung_scan3.cpp:1153-1161 prints it; returns the length (0 if cap is too small). */
size_t es_format_summary(const es_engine *engine, uint64_t lo, uint64_t hi, const es_counters *c,
                         char *buf, size_t cap);

/* Run-time schedule of the engine's kernels. Every schedule gives the same counters and
 * records; only the time differs. No reference counterpart (the reference's CPU loop has
 * nothing to schedule). */
typedef struct {
  uint32_t short_max;            /* windows whose lanes hold at most this many positions
                                    (1..es_info_t.short_max_limit, 128 in this build) go to the
                                    short-window kernel as they are; default the limit */
  uint32_t rung_blocks_per_sm;   /* stage-D grid in blocks per SM (1..16); default 6 */
  uint32_t long_split;           /* 1 (default): longer windows are cut into sub-windows of
                                    short_max positions per lane for the short-window kernel;
                                    0: they go to the segment marking */
  uint32_t reserved[5];          /* zero */
} es_schedule;

es_status es_get_schedule(const es_engine *engine, es_schedule *out);
/* ES_ERR_ARG for a value out of range; captured batch graphs are rebuilt on the next run. */
es_status es_set_schedule(es_engine *engine, const es_schedule *s);
/* Autotuner: runs the windows (persistent schedule) under each candidate schedule -- short_max
 * in {limit/4, limit/2, limit} x rung_blocks_per_sm in {4, 6, 8} x long_split in {1, 0} -- once to warm up
 * and `repeats` times
 * timed, keeps the mean device time of each, checks that every candidate gave identical
 * counters and records (ES_ERR_DEVICE_STATUS if not), and sets the fastest. `chosen` may be
 * null. */
es_status es_autotune(es_engine *engine, const es_window *w, size_t n, int repeats, es_schedule *chosen);

es_status es_info(const es_engine *engine, es_info_t *out);
/* The wheel classes in lane order (build_wheel, sieve/rung_scan3.cpp:211-226). */
es_status es_classes(const es_engine *engine, uint64_t *out, size_t cap);
es_status es_timing(const es_engine *engine, es_timing_t *out);
const char *es_status_str(es_status s);
const char *es_last_error(const es_engine *engine);

/* Device probes over caller arrays: the reference's per-prime functions, batched.
 * es_is_prime_batch: sprp2 && is_prime (sieve/rung_scan3.cpp:680-689,
 *   census/rung_scan.cpp:76-92); out[i] = 1 for a prime.
 * es_solve_rung_batch: solve_rung3 (sieve/rung_scan3.cpp:578-603); found[i] = 1 and
 *   out[i] filled (kind ES_REC_RUNG) when a rung certifies p[i].
 * es_solve_direct_batch: solve_direct3 (sieve/rung_scan3.cpp:624-647).
 * es_factor_batch: factorA_fast (sieve/rung_scan3.cpp:410-431); primes ascending,
 *   pr and ex hold 16 slots per value, k[i] the count. */
es_status es_is_prime_batch(es_engine *engine, const uint64_t *n, size_t count, uint8_t *out);
es_status es_solve_rung_batch(es_engine *engine, const uint64_t *p, size_t count, es_record *out,
                              uint8_t *found);
es_status es_solve_direct_batch(es_engine *engine, const uint64_t *p, size_t count, es_record *out,
                                uint8_t *found);
es_status es_factor_batch(es_engine *engine, const uint64_t *n, size_t count, uint64_t *pr,
                          uint8_t *ex, uint8_t *k);
/* Exact re-check of certificates on the device (the identity sieve/verify_covers.py:246-275
 * tests with rationals, in fixed-width integers): ok[i] = 1 when record i is a RUNG or SOLVED
 * certificate whose decomposition of 4/p holds, 0 otherwise (SURVIVOR records included). The
 * engine runs the same check on every certificate before emitting it; a failure there is
 * ES_ERR_DEVICE_STATUS ("certificate-self-check") and the certificate is not emitted. */
es_status es_check_records(es_engine *engine, const es_record *recs, size_t count, uint8_t *ok);

/* SHA-256 of a host buffer as 64 lowercase hex digits and a terminating NUL in out (cap >= 65);
 * returns 64, or 0 on a bad argument. Host only, no device needed: the digest a shard meta
 * records for its certificate stream (tools/run19.sh:70-77, `sha256sum`). */
size_t es_sha256_hex(const void *data, size_t n, char *out, size_t cap);

/* Primality of count values already on the device, for callers that cannot allocate
 * device memory (a process whose device memory is all reserved up front, code where an
 * allocation may not block or fail at run time, a framework that owns every allocation).
 * No counterpart in the reference, which has no device path of its own for this.
 * d_n and d_out are device pointers owned by the caller; out[i] = 1 when n[i] is prime
 * (the verdict of es_is_prime_batch). The work is queued on `stream` (a cudaStream_t; NULL
 * for the default stream) on the current device and the call returns without waiting.
 * Its scratch is a fixed array of (ES_NOALLOC_MAX + 64) 32-bit words in the library's
 * device image, held by every GPU that loads the library until the process exits; the call
 * itself allocates nothing. count above ES_NOALLOC_MAX is refused with ES_ERR_ARG. The first
 * call in a CUDA context (the device's primary context, and again after a cudaDeviceReset has
 * replaced it) looks up the array's device address (cudaGetSymbolAddress), so make it before
 * any stream capture. Every call shares the one array: calls that overlap on the GPU (on
 * different streams, or from different threads) race; serialise them. */
#define ES_NOALLOC_MAX (1u << 20)
es_status es_is_prime_noalloc(const uint64_t *d_n, size_t count, uint8_t *d_out, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* ES_SIEVE_H */
