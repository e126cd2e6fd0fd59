// es_cli.cpp -- rung_scan3_gb300: the reference scanner's command line over the GB300 engine.
//
// Same flags, refusals, exit codes and stdout record as sieve/rung_scan3.cpp:960-1163:
//   rung_scan3_gb300 LO HI [--mmax N] [--wheel M] [--seg N] [--threads N] [--shard i/n]
//                    [--progress N] [--filters FILE] [--sieve P] [--no-emit-survivors]
//                    [--no-rung]   (cover_scan's test hook: skip stage D, exercise stage E)
//   rung_scan3_gb300 --verify | --dump-classes [--wheel M] | --check-direct LO N
//                    | --check-factor [N]
// plus options of its own: --device N, --profile (stage timings on stderr), --autotune (time
// the engine's candidate schedules on the windows first and keep the fastest),
//   --meta FILE [--order round|lane] [--chunk-rounds R]
//                      the shard record of tools/run19.sh:70-77 instead of the stream: the
//                      stream is hashed as it is produced (certs=, cert_sha256=), SURVIVOR
//                      lines kept verbatim, SUMMARY last; stdout gets the SUMMARY only.
//                      --order round (default) emits the production driver's order
//                      (sieve/cuda/scan.cu:266-310: rounds of --seg positions, lanes in wheel
//                      order within a round), running the shard in chunks of R rounds (default
//                      64) so no chunk holds more than its own records; --order lane emits
//                      rung_scan3's order and runs the shard as one window.
//   --order round|lane without --meta: the stdout stream in that order (default lane, the
//                      order of rung_scan3; round is the production driver's, whose streams the
//                      published window digests are taken over). And
//   rung_scan3_gb300 --batch FILE [flags]   one "LO HI" per line, each window's stream and
//                                           SUMMARY in file order, run as one batch;
//   rung_scan3_gb300 --serve FILE|- [flags] the same lines read as they arrive (stdin for
//                                           "-"), each window submitted at once and printed in
//                                           input order as soon as it is done.
// stdout carries only the certificate stream and SUMMARY; everything else goes to stderr.
// Exit status: 0 no survivors, 2 survivors present, 1 refusal or error.
#include "../../include/es_sieve.h"
#include "es_digest.h"
#include "es_wheel.h"

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <cinttypes>
#include <ctime>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

typedef uint64_t u64;

static void print_records(FILE *out, const es_record *r, size_t n, bool emit_surv) {
  std::string buf;
  buf.reserve(1 << 20);
  char line[160];
  for (size_t i = 0; i < n; ++i) {
    if (!emit_surv && r[i].kind == ES_REC_SURVIVOR) continue;
    const size_t k = es_format_record(&r[i], line, sizeof line);
    buf.append(line, k);
    if (buf.size() > (1 << 20)) { fwrite(buf.data(), 1, buf.size(), out); buf.clear(); }
  }
  fwrite(buf.data(), 1, buf.size(), out);
}

// --serve: windows ("LO HI" per line) are read from FILE or standard input and submitted as
// they are read (es_submit: the engine batches whatever is queued whenever one of its
// serving streams frees up); each window's stream and SUMMARY go to stdout in input order as
// soon as it and every window before it are done. A full queue (ES_ERR_BUSY) makes the
// reader wait for the oldest window first.
static int serve_stream(es_engine *e, const char *path, const es_info_t &info, bool emit_surv) {
  FILE *in = strcmp(path, "-") ? fopen(path, "r") : stdin;
  if (!in) { fprintf(stderr, "FATAL: cannot open %s\n", path); return 1; }
  struct Pending { es_window w; uint64_t t; };
  std::deque<Pending> q;
  u64 survivors = 0;
  int rc = 0;
  auto finish_front = [&](int timeout_ms) -> es_status {   // prints the oldest window if done
    es_counters c;
    es_records r{};
    const es_status st = es_poll(e, q.front().t, &c, &r, timeout_ms);
    if (st == ES_ERR_TIMEOUT) return st;
    if (st != ES_OK) { fprintf(stderr, "FATAL: %s: %s\n", es_status_str(st), es_last_error(e)); return st; }
    print_records(stdout, r.recs, r.n, emit_surv);
    char line[512];
    fputs(es_format_summary(e, q.front().w.lo, q.front().w.hi, &c, line, sizeof line) ? line : "SUMMARY ?\n", stdout);
    fflush(stdout);
    survivors += c.survivors;
    es_free_records(&r);
    q.pop_front();
    return ES_OK;
  };
  unsigned long long a, b;
  while (rc == 0 && fscanf(in, "%llu %llu", &a, &b) == 2) {
    if (b > info.ceiling || a <= info.floor) {
      fprintf(stderr, "FATAL: window [%llu, %llu) outside (%llu, %llu]\n", a, b, (unsigned long long)info.floor,
              (unsigned long long)info.ceiling);
      rc = 1;
      break;
    }
    const es_window w{a, b};
    uint64_t t = 0;
    es_status st;
    while ((st = es_submit(e, &w, 1, &t)) == ES_ERR_BUSY && !q.empty())
      if (finish_front(-1) != ES_OK) { rc = 1; break; }
    if (rc) break;
    if (st != ES_OK) { fprintf(stderr, "FATAL: %s: %s\n", es_status_str(st), es_last_error(e)); rc = 1; break; }
    q.push_back({w, t});
    while (!q.empty()) {                             // print whatever is already done, in order
      const es_status f = finish_front(0);
      if (f == ES_ERR_TIMEOUT) break;
      if (f != ES_OK) { rc = 1; break; }
    }
  }
  while (rc == 0 && !q.empty())
    if (finish_front(-1) != ES_OK) rc = 1;
  if (in != stdin) fclose(in);
  return rc ? rc : (survivors ? 2 : 0);
}

static int open_engine(es_config &cfg, es_engine **e) {
  const es_status s = es_open(&cfg, e);
  if (s == ES_OK) return 0;
  if (s == ES_ERR_PIN) fprintf(stderr, "FATAL: %s\n", es_last_error(nullptr));
  else fprintf(stderr, "FATAL: engine: %s (%s)\n", es_status_str(s), es_last_error(nullptr));
  return 1;
}

static es_engine *default_engine(int device) {
  es_config cfg{};
  cfg.device = device;
  es_engine *e = nullptr;
  return open_engine(cfg, &e) ? nullptr : e;
}

// Walk the primes at or above lo on the device and run stage E on the first N
// (sieve/rung_scan3.cpp:798-817). Certificates to stdout, status to stderr.
static int check_direct(u64 lo, u64 N, int device) {
  es_engine *e = default_engine(device);
  if (!e) return 1;
  std::vector<u64> primes;
  const size_t chunk = 1 << 16;
  std::vector<u64> cand(chunk);
  std::vector<uint8_t> isp(chunk);
  u64 p = lo | 1ull;
  while (primes.size() < N) {
    for (size_t i = 0; i < chunk; ++i) cand[i] = p + 2 * i;
    if (es_is_prime_batch(e, cand.data(), chunk, isp.data()) != ES_OK) {
      fprintf(stderr, "FATAL: %s\n", es_last_error(e)); es_close(e); return 1;
    }
    for (size_t i = 0; i < chunk && primes.size() < N; ++i) if (isp[i]) primes.push_back(cand[i]);
    p += 2 * chunk;
  }
  std::vector<es_record> recs(N);
  std::vector<uint8_t> found(N);
  const es_status s = es_solve_direct_batch(e, primes.data(), N, recs.data(), found.data());
  if (s != ES_OK) { fprintf(stderr, "FATAL: %s\n", es_last_error(e)); es_close(e); return 1; }
  u64 solved = 0;
  char line[160];
  for (u64 i = 0; i < N; ++i) {
    if (found[i]) { ++solved; es_format_record(&recs[i], line, sizeof line); fputs(line, stdout); }
    else fprintf(stderr, "  stage E DECLINED p=%llu\n", (unsigned long long)primes[i]);
  }
  fprintf(stderr, "%s check-direct %llu/%llu primes at or above %llu solved by stage E (ceiling %llu)\n",
          solved == N ? "ok  " : "FAIL", (unsigned long long)solved, (unsigned long long)N,
          (unsigned long long)lo, (unsigned long long)es::DIRECT_PMAX);
  es_close(e);
  return solved == N ? 0 : 1;
}

// The adversarial factorization battery of sieve/rung_scan3.cpp:459-530, run on the device.
// Independent of any second factorizer: every product of prime powers must give back n,
// and every reported prime must pass the device Miller-Rabin.
static int check_factor(u64 nper, int device) {
  es_engine *e = default_engine(device);
  if (!e) return 1;
  u64 seed = 0x9e3779b97f4a7c15ull;
  auto rnd = [&]() { seed ^= seed << 13; seed ^= seed >> 7; seed ^= seed << 17; return seed; };
  auto next_prime = [&](u64 a) {   // smallest prime >= a, by device batches
    std::vector<u64> c(256);
    std::vector<uint8_t> f(256);
    for (;;) {
      for (int i = 0; i < 256; ++i) c[i] = a + (u64)i;
      es_is_prime_batch(e, c.data(), 256, f.data());
      for (int i = 0; i < 256; ++i) if (f[i]) return c[i];
      a += 256;
    }
  };
  const u64 NMAX = 18446744065119617025ull;
  std::vector<u64> vals;
  for (u64 dec = 1000000ull; dec < NMAX / 10; dec *= 10)
    for (u64 i = 0; i < nper; ++i) vals.push_back(dec + rnd() % (9 * dec));
  for (u64 i = 0; i < nper; ++i) {
    const u64 a = next_prime(3037000000ull + rnd() % 1257000000ull);
    const u64 b = next_prime(2147483648ull + rnd() % 2147000000ull);
    if ((unsigned __int128)a * b <= NMAX) vals.push_back(a * b);
  }
  for (u64 i = 0; i < nper; ++i) {
    const u64 a = next_prime(2147483648ull + rnd() % 2147000000ull);
    vals.push_back(a * a);
  }
  for (u64 i = 0; i < nper; ++i) {
    u64 v = 1;
    while (v < NMAX / 65536) v *= 2 + rnd() % 65535;
    vals.push_back(v);
  }
  for (u64 i = 0; i < nper / 4 + 1; ++i) vals.push_back(next_prime(((1ull << 62) + rnd() % (1ull << 62)) | 1ull));
  const u64 B = 65536ull * 65536ull;
  const u64 edge[] = {B - 1, B, B + 1, (1ull << 63) - 1, 1ull << 63, (1ull << 63) + 1, NMAX - 2, NMAX - 1, NMAX, 1, 2};
  for (u64 v : edge) vals.push_back(v);
  const size_t n = vals.size();
  std::vector<u64> pr(n * 16);
  std::vector<uint8_t> ex(n * 16), k(n);
  if (es_factor_batch(e, vals.data(), n, pr.data(), ex.data(), k.data()) != ES_OK) {
    fprintf(stderr, "FATAL: %s\n", es_last_error(e)); es_close(e); return 1;
  }
  std::vector<u64> facs;
  for (size_t i = 0; i < n; ++i) for (int j = 0; j < k[i]; ++j) facs.push_back(pr[i * 16 + j]);
  std::vector<uint8_t> fp(facs.size());
  if (!facs.empty()) es_is_prime_batch(e, facs.data(), facs.size(), fp.data());
  u64 bad_prod = 0, bad_prime = 0;
  for (size_t i = 0; i < n; ++i) {
    unsigned __int128 prod = 1;
    for (int j = 0; j < k[i]; ++j)
      for (int t = 0; t < ex[i * 16 + j]; ++t) prod *= pr[i * 16 + j];
    if (prod != (unsigned __int128)vals[i]) ++bad_prod;
  }
  for (uint8_t f : fp) if (!f) ++bad_prime;
  const u64 bad = bad_prod + bad_prime;
  printf("%s check-factor %zu values -- bad products: %llu, composite factors: %llu\n", bad ? "FAIL" : "ok  ", n,
         (unsigned long long)bad_prod, (unsigned long long)bad_prime);
  es_close(e);
  return bad ? 1 : 0;
}

static int self_test(int device) {
  std::string log;
  int fails = es::wheel_self_test(log);
  fputs(log.c_str(), stdout);
  // The device path: primality of known values, and one rung certificate.
  es_engine *e = default_engine(device);
  if (!e) { printf("  FAIL  device engine could not be opened\n"); ++fails; }
  else {
    const u64 v[6] = {2, 3037000493ull, 4611686018427387847ull, 18446744073709551557ull, 561, 3215031751ull};
    const uint8_t want[6] = {1, 1, 1, 1, 0, 0};
    uint8_t got[6] = {0};
    const bool ok = es_is_prime_batch(e, v, 6, got) == ES_OK && !memcmp(got, want, 6);
    printf(ok ? "  pass  %-50s = 6\n" : "  FAIL  %-50s\n", "device Miller-Rabin verdicts on known values");
    if (!ok) ++fails;
    es_close(e);
  }
  printf(fails ? "\nSELF-TEST FAILED (%d checks)\n" : "\nSELF-TEST PASSED\n", fails);
  return fails ? 1 : 0;
}

static std::string file_sha256(const char *path) {
  FILE *f = path ? fopen(path, "rb") : nullptr;
  if (!f) return "none";
  es::Sha256 h;
  std::vector<char> buf(1 << 16);
  size_t k;
  while ((k = fread(buf.data(), 1, buf.size(), f)) > 0) h.update(buf.data(), k);
  fclose(f);
  return h.hex();
}

// The shard record of tools/run19.sh:70-77 for [lo, hi): the stream is formatted and hashed
// chunk by chunk, never stored. Round order (sieve/cuda/scan.cu:266-310) needs each chunk to
// start on a round boundary of every lane: chunks are whole multiples of M * seg integers, so
// lane l's first position moves by exactly chunk_rounds * seg positions from one chunk to the
// next, and a stable counting sort of a chunk's lane-major records by J / seg gives round,
// lane, J. A producer thread keeps the GPU on the next chunk while this one is sorted,
// formatted by several threads and hashed in order.
// Records of one window (lane-major: lane, then J) put in the production driver's round-major
// order (round J / seg, then lane, then J) by a stable counting sort on the round.
static void sort_round_major(const es_record *rec, size_t n, u64 seg, std::vector<es_record> &out) {
  u64 rmax = 0;
  for (size_t i = 0; i < n; ++i) rmax = std::max<u64>(rmax, rec[i].J / seg);
  std::vector<size_t> start(rmax + 2, 0);
  for (size_t i = 0; i < n; ++i) ++start[rec[i].J / seg + 1];
  for (size_t k = 1; k < start.size(); ++k) start[k] += start[k - 1];
  out.resize(n);
  for (size_t i = 0; i < n; ++i) out[start[rec[i].J / seg]++] = rec[i];
}

struct Chunk {
  es_counters c{};
  es_records r{nullptr, 0};
  es_status st = ES_OK;
  bool last = false;
};

static int write_meta(es_engine *e, const char *path, u64 lo, u64 hi, u64 M, u64 seg, u64 chunk_rounds,
                      bool round_order, bool emit_surv, u64 shard, u64 nshard, const char *ffile, const char *threads,
                      std::chrono::steady_clock::time_point t0) {
  es::Sha256 h;
  u64 certs = 0;
  std::string surv_lines;
  es_counters tot{};
  const unsigned __int128 span128 = (unsigned __int128)M * seg * chunk_rounds;
  const u64 span = round_order && span128 < (unsigned __int128)(hi - lo) ? (u64)span128 : hi - lo;
  // producer: runs the chunks in order into a queue of at most two
  std::mutex mu;
  std::condition_variable cv;
  std::deque<Chunk> q;
  bool stop = false;
  std::thread prod([&] {
    for (u64 a = lo;;) {
      const u64 b = hi - a > span ? a + span : hi;
      Chunk ch;
      ch.st = es_run_window(e, a, b, &ch.c, &ch.r);
      ch.last = ch.st != ES_OK || b == hi;
      std::unique_lock<std::mutex> lk(mu);
      cv.wait(lk, [&] { return q.size() < 2 || stop; });
      if (stop) { es_free_records(&ch.r); return; }
      q.push_back(ch);
      cv.notify_all();
      if (ch.last) return;
      a = b;
    }
  });
  const unsigned nthr = std::max(1u, std::min(8u, std::thread::hardware_concurrency() / 2));
  std::vector<es_record> sorted;
  std::vector<std::string> text(nthr);
  std::vector<u64> tcerts(nthr);
  std::vector<std::string> tsurv(nthr);
  int rc = 0;
  for (;;) {
    Chunk ch;
    {
      std::unique_lock<std::mutex> lk(mu);
      cv.wait(lk, [&] { return !q.empty(); });
      ch = q.front();
      q.pop_front();
      cv.notify_all();
    }
    if (ch.st != ES_OK) {
      fprintf(stderr, "FATAL: %s: %s\n", es_status_str(ch.st), es_last_error(e));
      es_free_records(&ch.r);
      rc = 1;
      break;
    }
    const es_counters &c = ch.c;
    tot.positions += c.positions; tot.covered += c.covered; tot.sieved += c.sieved; tot.mr += c.mr;
    tot.composite += c.composite; tot.rung += c.rung; tot.direct += c.direct; tot.survivors += c.survivors;
    const es_record *rec = ch.r.recs;
    const size_t n = ch.r.n;
    if (round_order && n) {
      sort_round_major(rec, n, seg, sorted);
      rec = sorted.data();
    }
    std::vector<std::thread> pool;
    for (unsigned t = 0; t < nthr; ++t)
      pool.emplace_back([&, t] {
        const size_t a = n * t / nthr, b = n * (t + 1) / nthr;
        std::string &out = text[t];
        out.clear();
        out.reserve((b - a) * 80);
        tcerts[t] = 0;
        tsurv[t].clear();
        char line[192];
        for (size_t i = a; i < b; ++i) {
          if (!emit_surv && rec[i].kind == ES_REC_SURVIVOR) continue;
          const size_t k = es_format_record(&rec[i], line, sizeof line);
          out.append(line, k);
          if (rec[i].kind == ES_REC_SURVIVOR) tsurv[t].append(line, k);
          else ++tcerts[t];
        }
      });
    for (std::thread &t : pool) t.join();
    for (unsigned t = 0; t < nthr; ++t) {
      h.update(text[t]);
      certs += tcerts[t];
      surv_lines += tsurv[t];
    }
    es_free_records(&ch.r);
    if (ch.last) break;
  }
  {
    std::lock_guard<std::mutex> lk(mu);
    stop = true;
    cv.notify_all();
  }
  prod.join();
  for (Chunk &left : q) es_free_records(&left.r);
  if (rc) return rc;
  char summary[512];
  if (!es_format_summary(e, lo, hi, &tot, summary, sizeof summary)) { fprintf(stderr, "FATAL: SUMMARY\n"); return 1; }
  rc = tot.survivors ? 2 : 0;
  const long wall = (long)std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  char date[32];
  const time_t now = time(nullptr);
  strftime(date, sizeof date, "%Y-%m-%d %H:%M:%S", gmtime(&now));
  const std::string tmp = std::string(path) + ".tmp";
  FILE *f = fopen(tmp.c_str(), "w");
  if (!f) { fprintf(stderr, "FATAL: cannot write %s\n", tmp.c_str()); return 1; }
  fprintf(f, "# shard %llu/%llu  rc=%d  wall=%lds  attempt=1  %s\n", (unsigned long long)shard,
          (unsigned long long)nshard, rc, wall, date);
  fprintf(f, "# binary_commit=gb300 table_sha256=%s threads=%s order=%s\n", file_sha256(ffile).c_str(), threads,
          round_order ? "round" : "lane");
  fprintf(f, "certs=%llu\ncert_sha256=%s\n", (unsigned long long)certs, h.hex().c_str());
  fputs(surv_lines.c_str(), f);
  fputs(summary, f);                                   // last: its presence marks the meta complete
  if (fclose(f) != 0 || rename(tmp.c_str(), path) != 0) { fprintf(stderr, "FATAL: cannot write %s\n", path); return 1; }
  fputs(summary, stdout);
  return rc;
}

int main(int argc, char **argv) {
  int device = 0;
  for (int i = 1; i + 1 < argc; ++i) if (!strcmp(argv[i], "--device")) device = atoi(argv[i + 1]);
  if (argc >= 2 && !strcmp(argv[1], "--verify")) return self_test(device);
  if (argc >= 4 && !strcmp(argv[1], "--check-direct"))
    return check_direct(strtoull(argv[2], 0, 10), strtoull(argv[3], 0, 10), device);
  if (argc >= 2 && !strcmp(argv[1], "--check-factor"))
    return check_factor(argc >= 3 && argv[2][0] != '-' ? strtoull(argv[2], 0, 10) : 2000, device);
  if (argc >= 2 && !strcmp(argv[1], "--dump-classes")) {
    u64 dm = 2042040;
    for (int i = 2; i + 1 < argc; ++i) if (!strcmp(argv[i], "--wheel")) dm = strtoull(argv[i + 1], 0, 10);
    fputs(es::class_table_text(dm).c_str(), stdout);
    return 0;
  }
  const bool batch = argc >= 3 && !strcmp(argv[1], "--batch");
  const bool serve = argc >= 3 && !strcmp(argv[1], "--serve");
  if (argc < 3) {
    fprintf(stderr,
            "usage: %s LO HI [--mmax N] [--wheel M] [--seg N] [--threads N]\n"
            "                 [--shard i/n] [--progress N] [--filters FILE] [--sieve P]\n"
            "                 [--no-emit-survivors] [--device N] [--profile] [--autotune]\n"
            "                 [--meta FILE [--order round|lane] [--chunk-rounds R]]\n"
            "       %s --batch FILE [flags]\n"
            "       %s --serve FILE|- [flags]\n"
            "       %s --verify | --dump-classes [--wheel M] | --check-direct LO N | --check-factor [N]\n"
            "GB300 verification sieve: certifies 4/p solvable for every prime in [LO, HI),\n"
            "byte for byte the record of the reference rung_scan3.\n",
            argv[0], argv[0], argv[0], argv[0]);
    return 1;
  }
  u64 lo = 0, hi = 0;
  if (!batch && !serve) { lo = strtoull(argv[1], 0, 10); hi = strtoull(argv[2], 0, 10); }
  u64 M = 2042040, mmax = 10000, seg = 262144, shard = 0, nshard = 1, sieve_p = 0;
  bool emit_surv = true, profile = false, no_rung = false, autotune = false, round_order = true, order_given = false;
  const char *ffile = nullptr, *meta = nullptr, *threads = "1";
  u64 chunk_rounds = 64;
  for (int i = 3; i < argc; ++i) {
    if (!strcmp(argv[i], "--mmax") && i + 1 < argc) mmax = strtoull(argv[++i], 0, 10);
    else if (!strcmp(argv[i], "--wheel") && i + 1 < argc) M = strtoull(argv[++i], 0, 10);
    else if (!strcmp(argv[i], "--seg") && i + 1 < argc) seg = strtoull(argv[++i], 0, 10);
    else if (!strcmp(argv[i], "--progress") && i + 1 < argc) ++i;
    else if (!strcmp(argv[i], "--threads") && i + 1 < argc) threads = argv[++i];
    else if (!strcmp(argv[i], "--device") && i + 1 < argc) ++i;
    else if (!strcmp(argv[i], "--filters") && i + 1 < argc) ffile = argv[++i];
    else if (!strcmp(argv[i], "--sieve") && i + 1 < argc) sieve_p = strtoull(argv[++i], 0, 10);
    else if (!strcmp(argv[i], "--shard") && i + 1 < argc) {
      unsigned long long a = 0, b = 1;
      if (sscanf(argv[++i], "%llu/%llu", &a, &b) == 2) { shard = a; nshard = b; }
    } else if (!strcmp(argv[i], "--no-emit-survivors")) emit_surv = false;
    else if (!strcmp(argv[i], "--profile")) profile = true;
    else if (!strcmp(argv[i], "--no-rung")) no_rung = true;
    else if (!strcmp(argv[i], "--autotune")) autotune = true;
    else if (!strcmp(argv[i], "--meta") && i + 1 < argc) meta = argv[++i];
    else if (!strcmp(argv[i], "--chunk-rounds") && i + 1 < argc) chunk_rounds = strtoull(argv[++i], 0, 10);
    else if (!strcmp(argv[i], "--order") && i + 1 < argc) {
      const char *o = argv[++i];
      order_given = true;
      if (!strcmp(o, "round")) round_order = true;
      else if (!strcmp(o, "lane")) round_order = false;
      else { fprintf(stderr, "FATAL: --order must be round or lane\n"); return 1; }
    }
    else { fprintf(stderr, "FATAL: unknown option '%s'\n", argv[i]); return 1; }
  }
  if (!seg) seg = 262144;
  if (nshard == 0) nshard = 1;
  if (!chunk_rounds) chunk_rounds = 64;
  if (meta && (batch || serve)) {
    fprintf(stderr, "FATAL: --meta writes one shard's record; it does not take --batch or --serve\n");
    return 1;
  }
  if (!batch && !serve && nshard > 1) {       // ceil-span tiling, sieve/rung_scan3.cpp:1022-1027
    const u64 span = (hi - lo + nshard - 1) / nshard;
    const u64 a = lo + shard * span, b = std::min(hi, a + span);
    lo = a; hi = std::max(a, b);
  }
  uint64_t *fm = nullptr, *fr = nullptr;
  size_t nfil = 0;
  if (ffile) {
    const es_status s = es_load_filters(ffile, &fm, &fr, &nfil);
    if (s == ES_ERR_FILTERS) {
      FILE *t = fopen(ffile, "r");
      if (!t) fprintf(stderr, "FATAL: cannot open %s\n", ffile);
      else { fclose(t); fprintf(stderr, "FATAL: no FILTER lines in %s\n", ffile); }
      return 1;
    }
    if (s != ES_OK) { fprintf(stderr, "FATAL: %s\n", es_status_str(s)); return 1; }
  }
  es_config cfg{};
  cfg.wheel_M = M; cfg.mmax = mmax; cfg.sieve_p = sieve_p; cfg.seg = seg;
  cfg.filter_mods = fm; cfg.filter_ress = fr; cfg.n_filters = nfil; cfg.device = device;
  cfg.flags = no_rung ? ES_FLAG_NO_RUNG : 0;
  const auto t0 = std::chrono::steady_clock::now();
  es_engine *e = nullptr;
  if (open_engine(cfg, &e)) { es_free_u64(fm); es_free_u64(fr); return 1; }
  es_free_u64(fm); es_free_u64(fr);
  es_info_t info;
  es_info(e, &info);
  if (!info.pinned) fprintf(stderr, "[rung_scan3_gb300] WARNING: no pinned digest for M=%llu -- running UNPINNED\n",
                            (unsigned long long)M);
  if (serve) {
    const int rc = serve_stream(e, argv[2], info, emit_surv);
    es_close(e);
    return rc;
  }
  std::vector<es_window> wins;
  if (batch) {
    FILE *fp = fopen(argv[2], "r");
    if (!fp) { fprintf(stderr, "FATAL: cannot open %s\n", argv[2]); es_close(e); return 1; }
    unsigned long long a, b;
    while (fscanf(fp, "%llu %llu", &a, &b) == 2) wins.push_back({a, b});
    fclose(fp);
  } else {
    wins.push_back({lo, hi});
  }
  for (const es_window &w : wins) {
    if (w.hi > info.ceiling) {
      fprintf(stderr, "FATAL: HI must not exceed %llu, the stage-E ceiling: above it isqrt_u64 in the frozen "
                      "reference overflows, and a prime stage D misses would be reported as a survivor rather "
                      "than solved\n", (unsigned long long)info.ceiling);
      es_close(e);
      return 1;
    }
    if (w.lo <= info.floor) {
      fprintf(stderr, "FATAL: LO must exceed max pmin of the filter table (%llu); the region below is settled "
                      "by the existing censuses\n", (unsigned long long)info.floor);
      es_close(e);
      return 1;
    }
  }
  fprintf(stderr,
          "[rung_scan3_gb300] wheel M=%llu lanes=%llu (spacing %.0f)  covers=%llu (mmax=%llu)  seg=%llu  "
          "wheel_pmin=%llu\n[rung_scan3_gb300] filters=%llu fnv64=%016llx source=%s sieve=%llu (+%llu primes)\n",
          (unsigned long long)M, (unsigned long long)info.lanes, (double)M / (double)info.lanes,
          (unsigned long long)info.n_certified, (unsigned long long)mmax, (unsigned long long)seg,
          (unsigned long long)info.wheel_pmin, (unsigned long long)info.n_certified,
          (unsigned long long)info.filter_fnv64, ffile ? ffile : "generated", (unsigned long long)sieve_p,
          (unsigned long long)(info.n_filters - info.n_certified));
  if (autotune) {
    es_schedule sc;
    const es_status a = es_autotune(e, wins.data(), wins.size(), 6, &sc);
    if (a != ES_OK) {
      fprintf(stderr, "FATAL: autotune: %s: %s\n", es_status_str(a), es_last_error(e));
      es_close(e);
      return 1;
    }
    fprintf(stderr, "[rung_scan3_gb300] autotune: short_max=%u rung_blocks_per_sm=%u\n", sc.short_max,
            sc.rung_blocks_per_sm);
  }
  if (meta) {
    const int rc = write_meta(e, meta, lo, hi, M, seg, chunk_rounds, round_order, emit_surv, shard, nshard, ffile,
                              threads, t0);
    es_close(e);
    return rc;
  }
  const auto t1 = std::chrono::steady_clock::now();
  std::vector<es_counters> cnt(wins.size());
  es_records recs{};
  const es_status s = wins.size() == 1 ? es_run_window(e, wins[0].lo, wins[0].hi, &cnt[0], &recs)
                                       : es_run_batch(e, wins.data(), wins.size(), ES_SCHED_PERSISTENT, cnt.data(), &recs);
  if (s != ES_OK) {
    fprintf(stderr, "FATAL: %s: %s\n", es_status_str(s), es_last_error(e));
    es_close(e);
    return 1;
  }
  const auto t2 = std::chrono::steady_clock::now();
  u64 survivors = 0;
  size_t r0 = 0;
  std::vector<es_record> sorted;
  for (size_t w = 0; w < wins.size(); ++w) {
    size_t r1 = r0;
    while (r1 < recs.n && recs.recs[r1].window == w) ++r1;
    if (order_given && round_order) {              // the production driver's round-major order
      sort_round_major(recs.recs + r0, r1 - r0, seg, sorted);
      print_records(stdout, sorted.data(), sorted.size(), emit_surv);
    } else {
      print_records(stdout, recs.recs + r0, r1 - r0, emit_surv);
    }
    char line[512];
    fputs(es_format_summary(e, wins[w].lo, wins[w].hi, &cnt[w], line, sizeof line) ? line : "SUMMARY ?\n", stdout);
    survivors += cnt[w].survivors;
    r0 = r1;
  }
  fflush(stdout);
  if (profile) {
    es_timing_t t;
    es_timing(e, &t);
    fprintf(stderr,
            "[profile] setup=%.3fs run=%.3fs device_total=%.3fms mark=%.3fms mr=%.3fms rung=%.3fms direct=%.3fms "
            "items=%llu survivors=%llu primes=%llu launches=%llu\n",
            std::chrono::duration<double>(t1 - t0).count(), std::chrono::duration<double>(t2 - t1).count(),
            t.total_ms, t.mark_ms, t.mr_ms, t.rung_ms, t.direct_ms, (unsigned long long)t.mark_items,
            (unsigned long long)t.survivors, (unsigned long long)t.primes, (unsigned long long)t.kernel_launches);
  }
  es_free_records(&recs);
  es_close(e);
  return survivors ? 2 : 0;
}
