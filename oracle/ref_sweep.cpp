// ref_sweep.cpp -- in-process driver over the reference scanner's own sweep seam.
//
// TEST INFRASTRUCTURE ONLY (built by oracle/Makefile into oracle/_ref/, never shipped).
//
// It compiles sieve/rung_scan3.cpp from the reference tree with RUNG_SCAN3_NO_MAIN
// (sieve/rung_scan3.cpp:955-959) and calls its functions directly: gen_covers,
// gen_wheel_covers, gen_ucerts, build_wheel (:93-226), then sweep_lane (:711-784) per
// lane, merged strictly in lane order (:1146-1151), with the same SUMMARY line
// (:1153-1161). What it leaves out is the CLI's build_base_primes(hi) (:1073), which the
// sweep never reads and which costs minutes at 1.7e19. It is the reference arm for
// windows and window batches where the CLI's startup would swamp the measurement.
//
//   ref_sweep LO HI [--wheel M] [--mmax N] [--filters FILE] [--sieve P] [--threads T]
//             [--seg N] [--no-emit-survivors]
//   ref_sweep --windows FILE [same flags]     FILE: one "LO HI" per line; prints each
//                                             window's stream and SUMMARY in file order
// The sweep-only wall time goes to stderr as "sweep_seconds=<s>".
#define RUNG_SCAN3_NO_MAIN
#include "rung_scan3.cpp"
#include <chrono>

int main(int argc, char **argv) {
  if (argc < 3) { fprintf(stderr, "usage: ref_sweep LO HI [flags] | --windows FILE [flags]\n"); return 1; }
  vector<pair<u64, u64>> wins;
  int first_flag = 3;
  if (!strcmp(argv[1], "--windows")) {
    FILE *fp = fopen(argv[2], "r");
    if (!fp) { fprintf(stderr, "FATAL: cannot open %s\n", argv[2]); return 1; }
    unsigned long long a, b;
    while (fscanf(fp, "%llu %llu", &a, &b) == 2) wins.push_back({(u64)a, (u64)b});
    fclose(fp);
  } else {
    wins.push_back({strtoull(argv[1], 0, 10), strtoull(argv[2], 0, 10)});
  }
  u64 M = 2042040, mmax = 10000, seg = 262144, sieve_p = 0;
  int threads = 0; bool emit_surv = true; const char *ffile = nullptr;
  for (int i = first_flag; i < argc; ++i) {
    if (!strcmp(argv[i], "--wheel") && i + 1 < argc) M = strtoull(argv[++i], 0, 10);
    else if (!strcmp(argv[i], "--mmax") && i + 1 < argc) mmax = strtoull(argv[++i], 0, 10);
    else if (!strcmp(argv[i], "--seg") && i + 1 < argc) seg = strtoull(argv[++i], 0, 10);
    else if (!strcmp(argv[i], "--sieve") && i + 1 < argc) sieve_p = strtoull(argv[++i], 0, 10);
    else if (!strcmp(argv[i], "--threads") && i + 1 < argc) threads = atoi(argv[++i]);
    else if (!strcmp(argv[i], "--filters") && i + 1 < argc) ffile = argv[++i];
    else if (!strcmp(argv[i], "--no-emit-survivors")) emit_surv = false;
    else { fprintf(stderr, "FATAL: unknown option '%s'\n", argv[i]); return 1; }
  }
  const vector<Cover> covers = gen_covers(mmax);
  const WheelResult wr = build_wheel(M, gen_wheel_covers(M), gen_ucerts(UCERT_RMAX, UCERT_UMAX));
  const vector<u64> &wheel = wr.classes;
  u64 cover_pmax = 0;
  for (const Cover &f : covers) cover_pmax = max(cover_pmax, f.pmin);
  vector<u64> mods, ress;
  if (ffile) {
    FILE *fp = fopen(ffile, "r");
    if (!fp) { fprintf(stderr, "FATAL: cannot open %s\n", ffile); return 1; }
    char line[256];
    while (fgets(line, sizeof line, fp)) {
      unsigned long long mod, res;
      if (sscanf(line, "FILTER %llu %llu", &mod, &res) == 2) { mods.push_back(mod); ress.push_back(res); }
    }
    fclose(fp);
  } else {
    for (const Cover &f : covers) if (M % f.mod) { mods.push_back(f.mod); ress.push_back(f.res); }
  }
  const size_t ncov = mods.size();
  if (sieve_p) for (u64 q : small_primes(sieve_p, M)) { mods.push_back(q); ress.push_back(0); }
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#endif
  double total = 0;
  int rc = 0;
  for (auto [lo, hi] : wins) {
    if (hi > DIRECT_PMAX || lo <= max(wr.max_pmin, cover_pmax)) {
      fprintf(stderr, "FATAL: window [%" PRIu64 ",%" PRIu64 ") outside the floor/ceiling\n", lo, hi);
      return 1;
    }
    vector<Scan3Stats> lst(wheel.size());
    vector<vector<string>> lem(wheel.size());
    auto t0 = std::chrono::steady_clock::now();
#pragma omp parallel for schedule(dynamic, 1)
    for (size_t i = 0; i < wheel.size(); ++i)
      sweep_lane(wheel[i], lo, hi, M, mods, ress, ncov, seg, lst[i], lem[i]);
    total += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    Scan3Stats st;
    for (size_t i = 0; i < wheel.size(); ++i) {
      st.merge(lst[i]);
      for (const string &s : lem[i])
        if (emit_surv || s.compare(0, 9, "SURVIVOR ") != 0) fputs(s.c_str(), stdout);
    }
    printf("SUMMARY lo=%" PRIu64 " hi=%" PRIu64 " wheelM=%" PRIu64 " lanes=%zu mmax=%" PRIu64 " ucert_rmax=%" PRIu32 " "
           "ucert_umax=%" PRIu32 " wheel_pmin=%" PRIu64 " classes_sha256=%s positions=%" PRIu64 " "
           "covered=%" PRIu64 " sieved=%" PRIu64 " mr=%" PRIu64 " composite=%" PRIu64 " rung=%" PRIu64 " direct=%" PRIu64 " survivors=%" PRIu64 "\n",
           lo, hi, M, wheel.size(), mmax, UCERT_RMAX, UCERT_UMAX, wr.max_pmin,
           class_pin(M) ? class_pin(M)->sha256 : "unpinned", st.positions, st.covered, st.sieved,
           st.mr_calls, st.composite, st.rung_solved, st.direct_solved, st.survivors);
    if (st.survivors) rc = 2;
  }
  fprintf(stderr, "sweep_seconds=%.6f windows=%zu\n", total, wins.size());
  return rc;
}
