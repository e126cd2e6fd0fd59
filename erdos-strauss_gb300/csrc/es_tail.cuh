// es_tail.cuh -- warp-cooperative survivor tail: Miller-Rabin, factorization, the rung DP.
//
// One prime's rung walk is a chain of dependent steps (trial division, a primality test,
// sometimes Brent's rho, then a divisor DP), so a thread per prime is latency-bound: the
// slowest prime sets the time of the whole window. Here every step is spread over a warp:
//   trial division   lane i tests the odd primes i, i+32, ... below 2^16 against n by
//                    multiplicative inverse; hits are gathered by ballot and divided out of
//                    the cofactor with one warp-wide product of inverses per chunk
//   primality        lanes 0..11 each run one of the 12 strong-probable-prime rounds
//   Brent's rho      all 32 lanes walk with different constants c; the first split wins
//                    (the factorization is unique, so which lane wins cannot change it)
//   ECM              in the latency-bound tail, a cofactor rho has not split after ECM_AFTER
//                    steps gets rounds of one elliptic curve per lane (es_ecm.cuh), the first
//                    divisor wins
//   rung DP          lanes own residue classes t mod r and gather
//                    nxt[t] = min_j cur[t * pr^-j] * pr^j over j <= e with the bound <= q
// and a block of four warps walks successive rungs of one prime concurrently, keeping the
// smallest rung that certifies (the reference's emission rule, sieve/rung_scan3.cpp:574-603).
#pragma once
#include "es_arith.cuh"
#include "es_ecm.cuh"

namespace es {

constexpr unsigned FULL = 0xFFFFFFFFu;
constexpr int TD_CHUNKS = (NTD + 31) / 32;     // 205 chunks of 32 primes
constexpr u64 WARP_RHO_STEPS = 1ull << 24;     // per lane, per split

struct WarpFac {          // shared memory, one per warp
  u64 pr[MAXF];
  u32 ex[MAXF];
  int k;
  int overflow;
};

// Append prime p with exponent e (merging a repeat). Lane 0 writes; all lanes call.
__device__ __forceinline__ void wf_add(WarpFac &F, u64 p, int e, u32 lane) {
  if (lane == 0) {
    int i = 0;
    for (; i < F.k; ++i) if (F.pr[i] == p) { F.ex[i] += e; break; }
    if (i == F.k) {
      if (F.k < MAXF) { F.pr[F.k] = p; F.ex[F.k] = e; ++F.k; } else F.overflow = 1;
    }
  }
  __syncwarp();
}

// The 12-base deterministic test (census/rung_scan.cpp:76-92) with one base per lane.
// All lanes must call; returns the same verdict in every lane.
__device__ inline bool warp_is_prime(u64 n, u32 lane) {
  bool ok = true;
  if (n < 2) return false;
  if (n <= 37) {
    bool isb = false;
    #pragma unroll
    for (int i = 0; i < 12; ++i) isb |= (n == MR_BASES[i]);
    return isb;
  }
  if (lane < 12) {
    const u64 b = MR_BASES[lane];
    if (n % b == 0) ok = false;
    else {
      const Mont M = mont_init(n);
      u64 d = n - 1;
      const int s = __ffsll((long long)d) - 1;
      d >>= s;
      const u64 bm = to_mont(b, M);
      ok = n < LazyArith::NMAX ? sprp_ar<LazyArith>(bm, d, s, M) : sprp_mont(bm, d, s, M);
    }
  }
  return __all_sync(FULL, ok);
}

// Brent's backtrack from ys: step one at a time until gcd(|x - ys|, n) > 1 (bounded by the
// longest batch).
constexpr u32 RHO_BATCH_MAX_BACKTRACK = 512;
template <class Ar>
__device__ __forceinline__ u64 rho_backtrack(u64 x, u64 ys, u64 cm, u64 n, const Mont &M) {
  u64 g = 1;
  for (u32 guard = 0; g == 1 && guard <= RHO_BATCH_MAX_BACKTRACK; ++guard) {
    ys = Ar::add(Ar::mul(ys, ys, M), cm, M);
    const u64 diff = x > ys ? x - ys : ys - x;
    g = gcd64(diff ? diff : n, n);
  }
  return g;
}

// Brent's rho, one walk per lane (constants c = 1 + lane + 32j for successive tries): the
// schedule of sieve/rung_scan3.cpp:333-369 -- y -> y^2 + c in Montgomery form, products of
// |x - y| accumulated between gcds, the comparison window doubling -- with two changes that
// cannot change a result, only when a factor is found: the first window is 16 steps instead
// of 1 (every cofactor that reaches rho has all its primes above 2^16, so its cycles are far
// longer) and gcds come every 256 steps instead of 128 (a 64-bit binary gcd costs about as
// much as twenty steps here). A 64-bit Montgomery multiply is issue-bound on this GPU (the
// wide integer multiplies issue at a quarter of the low-half rate), so more walks per lane
// would only add work: the latency-optimal split is one walk per lane.
// The lanes run in lockstep (one window schedule for the warp), so that the warp can stop as
// soon as any lane has a divisor, poll the hard board between batches and be cancelled
// there. A lane whose batch product shares all of n backtracks one step at a time from the
// batch start; if that closes without a divisor its walk restarts with its next constant.
// Returns a nontrivial factor of the odd composite n (the same value in every lane), or 0
// when the budget ran out or the warp was cancelled. The factorization is unique, so which
// walk wins cannot change any result.
constexpr u64 RHO_R0 = 16;      // first comparison window
constexpr u64 RHO_BATCH = 256;  // steps between gcds

// cancel/my_k: the warp is working for rung index my_k of a block whose best certifying rung
// so far is *cancel; once that drops below my_k nothing this warp finds can matter and it stops
// (returning 0 without an error). cancel may be null.
__device__ __forceinline__ bool cancelled(const volatile int *cancel, int my_k) {
  return cancel && *cancel < my_k;
}

// The hard board: a cofactor that rho has not split in its first steps is posted here when its
// owner turns to ECM, and warps with nothing left to do (k_rung blocks that found the prime
// queue empty) run more rho walks on it with constants of their own. Any nontrivial divisor
// ends the search; by the birthday bound the wait for the first collision among W walks
// shrinks like 1/sqrt(W), so with hundreds of idle warps the helpers' walks can beat the
// owner's fixed-length ECM round, while a cofactor left alone gets the ECM round. The board
// only speeds things up: the owner checks every divisor it is handed (1 < d < n,
// n mod d == 0) and its own curves and walks still finish the job alone. No warp ever waits
// for another.
constexpr u32 HARD_SLOTS = 32;                 // one per lane of a scanning warp
#ifndef ES_RHO_POST_STEPS
#define ES_RHO_POST_STEPS 512
#endif
#ifndef ES_HELP_R0
#define ES_HELP_R0 16
#endif
#ifndef ES_HELP_SLEEP_NS
#define ES_HELP_SLEEP_NS 2000
#endif
constexpr u64 RHO_POST_STEPS = ES_RHO_POST_STEPS;  // steps per lane before a cofactor is posted
constexpr u64 HELP_STEPS = 1ull << 16;         // steps per lane of one helping session
constexpr u32 HELP_IDLE_POLLS = 4096;          // empty-board polls (2 us apart) before a helper leaves
constexpr u32 HELP_MAX_ROUNDS = 1024;          // board scans (sessions or polls) per helper, at most
struct HardSlot {
  unsigned long long n, found;
  unsigned int state, pad;                     // 0 free, 1 being written, 2 posted
  unsigned long long pad2;
};
// A block's own hard cofactor (shared memory): when a warp of a block that works on one
// prime's rungs has walked rho on a cofactor for RHO_POST_STEPS steps, it posts the cofactor
// here; block-mates that have finished their own rungs run rounds of elliptic curves on it
// instead of waiting at the block's barrier, and the first divisor found ends the search.
struct BlockHelp {
  unsigned long long n, found;                 // the posted cofactor (0: none), a divisor of it
  unsigned int busy;                           // warps of the block still on their rungs
  unsigned int sessions;                       // curve rounds started on the block's cofactors
};
struct HardBoard {
  HardSlot *slot;                              // [HARD_SLOTS], all free between runs
  unsigned long long *sessions;                // helping sessions started (distinct constants)
  unsigned long long *done;                    // primes finished by k_rung
  unsigned long long total;                    // primes k_rung has to finish
  BlockHelp *local;                            // the block's own slot, or null
  u64 ecm_after;                               // rho steps per lane before curves (0: ECM_AFTER)
};

__device__ __forceinline__ u64 ld_volatile(const unsigned long long *p) { return *(const volatile unsigned long long *)p; }
__device__ __forceinline__ u32 ld_volatile(const unsigned int *p) { return *(const volatile unsigned int *)p; }

// The lockstep walk shared by the owner and its helpers. c0: this lane's first constant,
// cstep: the distance to its next one. poll() is called by every lane between batches (warp-
// uniform) and returns a divisor handed in from outside, ~0 to stop, or 0 to go on. Ar is the
// arithmetic (es_arith.cuh): LazyArith for n < 2^62, ExactArith above.
template <class Ar, class Poll>
__device__ __forceinline__ u64 rho_walk(u64 n, const Mont &M, u64 c0, u64 cstep, u64 budget, u32 lane, Poll poll,
                                        u64 r0 = RHO_R0) {
  const u64 y0 = to_mont(2, M);
  u64 c = c0;
  u64 cm = to_mont(c, M);
  u64 y = y0, x = y0, ys = y0, q = M.one;
  u64 steps = 0;
  for (u64 r = r0;; r <<= 1) {
    x = y;
    if (steps + 2 * r > budget) return 0;
    for (u64 i = 0; i < r; ++i) y = Ar::add(Ar::mul(y, y, M), cm, M);
    steps += r;
    for (u64 k = 0; k < r; k += RHO_BATCH) {
      ys = y;
      const u64 lim = RHO_BATCH < r - k ? RHO_BATCH : r - k;
      for (u64 i = 0; i < lim; ++i) {
        y = Ar::add(Ar::mul(y, y, M), cm, M);
        q = Ar::mul(q, x > y ? x - y : y - x, M);     // a closed cycle makes q = 0 mod n
      }
      steps += lim;
      u64 mine = 0;
      const u64 g = gcd64(q, n);
      if (g != 1) {
        if (g != n) mine = g;
        else {
          const u64 gb = rho_backtrack<Ar>(x, ys, cm, n, M);
          if (gb != 1 && gb != n) mine = gb;
          else {                                        // this walk is spent: next constant
            c += cstep;
            cm = to_mont(c, M);
            y = y0; x = y0; q = M.one;
          }
        }
      }
      const unsigned has = __ballot_sync(FULL, mine != 0);
      if (has) return __shfl_sync(FULL, mine, __ffs(has) - 1);
      const u64 ext = poll(steps);
      if (ext) return ext == ~0ull ? 0 : ext;
    }
  }
}

// One round of elliptic curves on n, one per lane: lane l takes sigma0 + l. poll()
// returns what rho_walk's does (a divisor handed in, ~0 to stop, 0 to go on); a nonzero answer
// ends the round and is left in ext. Returns the first divisor a lane found (the same value in
// every lane), or 0.
template <class Ar, class Poll>
__device__ inline u64 warp_ecm(const Mont &M, u64 sigma0, u32 lane, Poll poll, u64 &ext) {
  ext = 0;
  auto p = [&]() -> bool { ext = poll(); return ext != 0; };
  const u64 d = ecm_curve<Ar>(sigma0 + lane, M, p);
  const unsigned has = __ballot_sync(FULL, d != 0);
  return has ? __shfl_sync(FULL, d, __ffs(has) - 1) : 0;
}

// Rho steps per lane before a cofactor goes to ECM: rho is the cheaper method for a prime
// factor below ~2^22 (its expected walk over 32 lanes is a few hundred steps), ECM above.
#ifndef ES_ECM_AFTER
#define ES_ECM_AFTER 512
#endif
constexpr u64 ECM_AFTER = ES_ECM_AFTER;
constexpr u32 ECM_OWNER_ROUNDS = 32;     // 1024 curves: a 31-bit factor survives them w.p. ~2e-7
constexpr u64 ECM_SIGMA_OWNER = 6;       // owner round r: sigma = 6 + 32 r + lane
constexpr u64 ECM_SIGMA_HELP = 4096;     // helper session t: sigma = 4096 + 32 t + lane
constexpr u64 ECM_SIGMA_LOCAL = 1ull << 22;   // block-mate session t: sigma = 2^22 + 32 t + lane
constexpr u32 LOCAL_HELP_POLLS = 1u << 16;   // empty-slot polls (0.5 us apart) before a block-mate stops
constexpr u32 LOCAL_HELP_ROUNDS = 1u << 12;  // curve rounds per block-mate and prime, at most
#ifndef ES_LOCAL_HELP
#define ES_LOCAL_HELP 1
#endif
// Helpers on the hard board run rounds of curves (1) or Brent walks (0).
#ifndef ES_HELP_ECM
#define ES_HELP_ECM 0
#endif

__device__ inline u64 warp_rho(u64 n, u32 lane, volatile u64 *found, u32 *status, const volatile int *cancel = nullptr,
                               int my_k = 0, const HardBoard *board = nullptr, u64 budget = WARP_RHO_STEPS,
                               bool use_ecm = true) {
  const Mont M = mont_init(n);
  int slot = -1;                                   // the board slot this warp posted n in
  bool local_posted = false;                       // n is in the block's own slot
  bool stop = false;                               // cancelled (warp-uniform)
  BlockHelp *const bh = board ? board->local : nullptr;
  auto poll = [&](u64 steps) -> u64 {
    u64 ext = 0;
    if (lane == 0 && bh) {
      if (!local_posted && steps >= RHO_POST_STEPS && n < LazyArith::NMAX) {
        local_posted = atomicCAS(&bh->n, 0ull, (unsigned long long)n) == 0ull;
        if (local_posted) *(volatile unsigned long long *)&bh->found = 0;   // no divisor of an earlier one
      }
      if (local_posted) {
        const u64 d = *(volatile unsigned long long *)&bh->found;
        if (d > 1 && d < n && n % d == 0) ext = d;
      }
    }
    if (lane == 0 && !ext) {
      if (cancelled(cancel, my_k)) ext = ~0ull;
      else if (board && slot < 0 && steps >= RHO_POST_STEPS) {
        for (u32 j = 0; j < HARD_SLOTS; ++j)
          if (atomicCAS(&board->slot[j].state, 0u, 1u) == 0u) {
            board->slot[j].n = n;
            board->slot[j].found = 0;
            __threadfence();
            atomicExch(&board->slot[j].state, 2u);
            slot = (int)j;
            break;
          }
        if (slot < 0) slot = (int)HARD_SLOTS;      // board full: do not try again
      } else if (board && slot >= 0 && slot < (int)HARD_SLOTS) {
        const u64 d = ld_volatile(&board->slot[slot].found);
        if (d > 1 && d < n && n % d == 0) ext = d;
      }
    }
    ext = __shfl_sync(FULL, ext, 0);
    if (ext == ~0ull) stop = true;
    return ext;
  };
  // Brent's rho first; a cofactor it has not split goes to ECM rounds (charged against the same
  // budget), and rho resumes with fresh constants for whatever budget remains after them. Every
  // stage-D cofactor is below 2^62 (A = (p + r)/4 with p below 2^64) and takes the lazy
  // arithmetic; larger n (factorization probes only) walk rho in exact arithmetic, without ECM.
  u64 f = 0;
  if (n >= LazyArith::NMAX) {
    f = rho_walk<ExactArith>(n, M, 1 + lane, 32, budget, lane, poll);
  } else {
    const u64 after = board && board->ecm_after ? board->ecm_after : ECM_AFTER;
    const bool ecm = use_ecm && budget >= after + ECM_ROUND_STEPS;
    f = rho_walk<LazyArith>(n, M, 1 + lane, 32, ecm ? after : budget, lane, poll);
    if (!f && !stop && ecm) {
      u64 steps = after;
      u64 ext = poll(RHO_POST_STEPS > steps ? RHO_POST_STEPS : steps);   // post n to the board now
      if (ext && ext != ~0ull) f = ext;
      for (u32 round = 0; !f && !stop && round < ECM_OWNER_ROUNDS && steps + ECM_ROUND_STEPS <= budget; ++round) {
        f = warp_ecm<LazyArith>(M, ECM_SIGMA_OWNER + 32 * (u64)round, lane, [&]() -> u64 { return poll(steps); }, ext);
        steps += ECM_ROUND_STEPS;
        if (!f && ext && ext != ~0ull) f = ext;
      }
      if (!f && !stop && steps < budget)
        f = rho_walk<LazyArith>(n, M, 1 + lane + 32 * 1024, 32, budget - steps, lane, poll);
    }
  }
  if (lane == 0 && local_posted) {                 // take n out of the block's slot
    *(volatile unsigned long long *)&bh->found = 0;
    __threadfence_block();
    atomicExch(&bh->n, 0ull);
  }
  if (lane == 0 && slot >= 0 && slot < (int)HARD_SLOTS) {  // take n off the board
    atomicExch(&board->slot[slot].state, 1u);
    board->slot[slot].n = 0;
    board->slot[slot].found = 0;
    __threadfence();
    atomicExch(&board->slot[slot].state, 0u);
  }
  if (lane == 0) *found = f;
  __syncwarp();
  if (!f && lane == 0 && !cancelled(cancel, my_k)) atomicOr(status, ST_RHO_BUDGET);
  return f;
}

// One helping pass of a warp with nothing else to do: pick a posted cofactor, walk HELP_STEPS
// steps per lane with constants no other walk uses (or run a round of curves, with ecm), and
// post the first divisor found. Returns 2 when every prime of the run is finished, 0 when the
// board was empty, 1 otherwise. All lanes call.
__device__ inline int warp_help_once(const HardBoard &B, u32 lane, bool ecm) {
  if (ld_volatile(B.done) >= B.total) return 2;
  const u32 st = lane < HARD_SLOTS ? ld_volatile(&B.slot[lane].state) : 0u;
  const unsigned posted = __ballot_sync(FULL, st == 2u);
  if (!posted) return 0;
  u64 ses = 0;
  if (lane == 0) ses = atomicAdd(B.sessions, 1ull);
  ses = __shfl_sync(FULL, ses, 0);
  u32 pick = (u32)(ses % (u64)__popc(posted)), j = 0;
  for (unsigned m = posted;; m &= m - 1) {
    if (pick-- == 0) { j = (u32)(__ffs(m) - 1); break; }
  }
  HardSlot *hs = &B.slot[j];
  const u64 n = ld_volatile(&hs->n);
  __threadfence();
  if (ld_volatile(&hs->state) != 2u || n <= 0xFFFFFFFFull || !(n & 1)) return 1;
  const Mont M = mont_init(n);
  auto poll = [&](u64) -> u64 {
    u64 ext = 0;
    if (lane == 0)
      ext = (ld_volatile(&hs->state) != 2u || ld_volatile(&hs->n) != n || ld_volatile(&hs->found) != 0) ? ~0ull : 0;
    return __shfl_sync(FULL, ext, 0);
  };
  // A round of curves polls its slot every few ladder bits and every few giant steps, so it
  // stops as soon as the cofactor is split; its sigmas lie above every owner's (an owner's round
  // r uses 6 + 32 r + lane, r < ECM_OWNER_ROUNDS) and are distinct per session. Rho walks take
  // constants above every owner's (an owner walks c = 1 + lane + 32 j with j below 2^12),
  // distinct per session (2^20 sessions apart before a restart adds 2^25); a posted cofactor has
  // already outlasted its owner's first walks, so helpers start with a longer window.
  u64 d = 0;
  if (ecm && n < LazyArith::NMAX) {
    u64 ext = 0;
    d = warp_ecm<LazyArith>(M, ECM_SIGMA_HELP + 32 * (ses & 0xFFFFFull), lane, [&]() -> u64 { return poll(0); },
                            ext);
  } else {
    const u64 c0 = (1ull << 24) + 32 * (ses & 0xFFFFFull) + 1 + lane;
    d = n < LazyArith::NMAX ? rho_walk<LazyArith>(n, M, c0, 1ull << 25, HELP_STEPS, lane, poll, ES_HELP_R0)
                            : rho_walk<ExactArith>(n, M, c0, 1ull << 25, HELP_STEPS, lane, poll, ES_HELP_R0);
  }
  if (lane == 0 && d > 1 && d < n && n % d == 0 && ld_volatile(&hs->n) == n)
    atomicCAS(&hs->found, 0ull, (unsigned long long)d);
  __syncwarp();
  return 1;
}

// A warp with nothing left to do helps the posted cofactors until every prime of the run is
// finished (or the board stays empty for HELP_IDLE_POLLS polls, or after HELP_MAX_ROUNDS
// sessions). All lanes call.
__device__ inline void warp_help(const HardBoard &B, u32 lane) {
  for (u32 idle = 0, round = 0; idle < HELP_IDLE_POLLS && round < HELP_MAX_ROUNDS + HELP_IDLE_POLLS; ++round) {
    const int h = warp_help_once(B, lane, ES_HELP_ECM);
    if (h == 2) return;
    if (h == 0) {
      ++idle;
      __nanosleep(ES_HELP_SLEEP_NS);
    }
  }
}

// A warp that has finished its rungs helps the block's posted cofactor until every warp of the
// block has finished: rounds of curves with sigmas of their own (2^22 + 32 t + lane, t the
// block's session count), each polling the slot every few ladder bits so that it stops as soon
// as the cofactor is split or withdrawn. Bounded: LOCAL_HELP_POLLS empty polls at most, and
// every round is bounded. All lanes call.
__device__ inline void warp_help_block(BlockHelp *bh, u32 lane) {
  for (u32 idle = 0, rounds = 0; idle < LOCAL_HELP_POLLS && rounds < LOCAL_HELP_ROUNDS;) {
    u64 n = 0, found = 0;
    u32 busy = 0;
    if (lane == 0) {
      busy = *(volatile unsigned int *)&bh->busy;
      n = *(volatile unsigned long long *)&bh->n;
      found = *(volatile unsigned long long *)&bh->found;
    }
    busy = __shfl_sync(FULL, busy, 0);
    if (!busy) return;
    n = __shfl_sync(FULL, n, 0);
    found = __shfl_sync(FULL, found, 0);
    if (!n || found || n >= LazyArith::NMAX || !(n & 1)) { ++idle; __nanosleep(500); continue; }
    ++rounds;
    u32 ses = 0;
    if (lane == 0) ses = atomicAdd(&bh->sessions, 1u);
    ses = __shfl_sync(FULL, ses, 0);
    const Mont M = mont_init(n);
    auto poll = [&]() -> u64 {
      u64 stop = 0;
      if (lane == 0)
        stop = (*(volatile unsigned long long *)&bh->n != n || *(volatile unsigned long long *)&bh->found != 0 ||
                *(volatile unsigned int *)&bh->busy == 0) ? ~0ull : 0;
      return __shfl_sync(FULL, stop, 0);
    };
    u64 ext = 0;
    const u64 d = warp_ecm<LazyArith>(M, ECM_SIGMA_LOCAL + 32 * (u64)ses, lane, poll, ext);
    if (lane == 0 && d > 1 && d < n && n % d == 0 && *(volatile unsigned long long *)&bh->n == n)
      atomicCAS(&bh->found, 0ull, (unsigned long long)d);
    __syncwarp();
  }
}

// The prime factors of a cofactor v > 2^32 with no prime factor below 2^16 (so at most three
// of them), appended to F: primes and squares at once, anything else split by warp_rho. All
// lanes call. Returns false when a bound was hit (status says which) or on cancellation.
__device__ inline bool warp_factor_cofactor(u64 v0, WarpFac &F, u32 *status, u32 lane, volatile u64 *rho_slot,
                                            const volatile int *cancel, int my_k, const HardBoard *board,
                                            u64 rho_budget, bool use_ecm) {
  u64 stack[4];
  int sp = 0;
  stack[sp++] = v0;
  for (int guard = 0; sp > 0; ++guard) {
    if (guard > 16) { if (lane == 0) atomicOr(status, ST_STACK_OVERFLOW); return false; }
    const u64 v = stack[--sp];
    if (v == 1) continue;
    if (cancel && __shfl_sync(FULL, cancelled(cancel, my_k) ? 1 : 0, 0)) return false;
    if (v <= 0xFFFFFFFFull || warp_is_prime(v, lane)) { wf_add(F, v, 1, lane); continue; }
    const u64 s = isqrt64(v);
    if (s * s == v) { wf_add(F, s, 2, lane); continue; }
    const u64 d = warp_rho(v, lane, rho_slot, status, cancel, my_k, board, rho_budget, use_ecm);
    if (d == 0) return false;                  // budget (status set) or cancelled
    if (sp + 2 > 4) { if (lane == 0) atomicOr(status, ST_STACK_OVERFLOW); return false; }
    stack[sp++] = d;
    stack[sp++] = v / d;
  }
  __syncwarp();
  if (F.overflow) { if (lane == 0) atomicOr(status, ST_FAC_OVERFLOW); return false; }
  return true;
}

// The odd primes below 2^16 dividing each rung of one prime, found for all rungs at once:
// rung k's A is A_k = floor(p/4) + 1 + k (A = (p + r)/4 with r = r0 + 4k and p + r0 = 4
// floor(p/4) + 4), so q | A_k exactly when k = -A_0 (mod q), and one residue A_0 mod q per
// prime q replaces trial division of every rung by q. The 17 primes below TD_RUNGS divide many
// rungs each and are kept as a bit mask per rung; every larger prime divides at most one of
// the 64 rungs and goes into that rung's list. Rung k then divides out only its own primes; a
// list longer than TD_LIST_CAP is marked incomplete and that rung trial-divides.
constexpr int TD_RUNGS = 64;            // rung indices 0 .. 63 (r = r0 + 4k <= RCAP)
constexpr int TD_SMALL = 17;            // odd primes below TD_RUNGS: 3 .. 61, tdp[0 .. 16]
constexpr int TD_LIST_CAP = 15;         // with TD_SMALL, at most 32: one prime per lane
struct TdSieve {                        // shared memory, one per block
  u16 idx[TD_RUNGS][TD_LIST_CAP];       // indices into tdp of the primes above 61 dividing A_k
  u32 n[TD_RUNGS];                      // their count (above TD_LIST_CAP: the list is incomplete)
  u32 small[TD_RUNGS];                  // bit i: tdp[i] divides A_k, i < TD_SMALL
  uint2 qm[TD_SMALL];                   // tdp[i] and floor(2^32 / tdp[i])
  u32 rs[TD_SMALL];                     // A_0 mod tdp[i]
};

// x mod q for x < 2^32 and an odd prime q < 2^16, m = floor(2^32 / q) (Barrett: the
// quotient estimate umulhi(x, m) is low by at most one).
__device__ __forceinline__ u32 mod_q16(u32 x, u32 q, u32 m) {
  const u32 r = x - __umulhi(x, m) * q;
  return r >= q ? r - q : r;
}
__device__ __forceinline__ u32 mod_a0(u32 hi, u32 mid, u32 lo, u32 q, u32 m) {   // A0 mod q, 16 bits at a time
  u32 r = mod_q16(hi, q, m);
  r = mod_q16((r << 16) | mid, q, m);
  return mod_q16((r << 16) | lo, q, m);
}

// S for A_k = A0 + k, k < TD_RUNGS, A0 < 2^64, from tdqm[i] = {d_i, floor(2^32 / d_i)} over
// the odd primes d_i below 2^16. Each thread takes SIEVE_BATCH primes at a time, their table
// entries loaded together before any is used. Every thread of the block calls; the block
// synchronizes on entry and exit.
constexpr int SIEVE_BATCH = 8;
__device__ inline void block_td_sieve(u64 A0, const uint2 *__restrict__ tdqm, TdSieve &S) {
  const u32 hi = (u32)(A0 >> 32), mid = (u32)(A0 >> 16) & 0xFFFFu, lo = (u32)A0 & 0xFFFFu;
  for (int k = threadIdx.x; k < TD_RUNGS; k += blockDim.x) S.n[k] = 0;
  if (threadIdx.x < TD_SMALL) {
    const uint2 e = __ldg(tdqm + threadIdx.x);
    S.qm[threadIdx.x] = e;
    S.rs[threadIdx.x] = mod_a0(hi, mid, lo, e.x, e.y);
  }
  __syncthreads();
  for (int k = threadIdx.x; k < TD_RUNGS; k += blockDim.x) {   // the small primes, rung by rung
    u32 mask = 0;
    #pragma unroll
    for (int i = 0; i < TD_SMALL; ++i) {
      const uint2 e = S.qm[i];
      if (mod_q16(S.rs[i] + (u32)k, e.x, e.y) == 0) mask |= 1u << i;
    }
    S.small[k] = mask;
  }
  for (int i0 = TD_SMALL + threadIdx.x; i0 < NTD; i0 += SIEVE_BATCH * blockDim.x) {
    uint2 e[SIEVE_BATCH];
    #pragma unroll
    for (int j = 0; j < SIEVE_BATCH; ++j) {
      const int i = i0 + j * (int)blockDim.x;
      e[j] = i < NTD ? __ldg(tdqm + i) : make_uint2(0u, 0u);
    }
    #pragma unroll
    for (int j = 0; j < SIEVE_BATCH; ++j) {
      if (!e[j].x) continue;
      const u32 r = mod_a0(hi, mid, lo, e[j].x, e[j].y);
      const u32 k = r ? e[j].x - r : 0u;                 // q > TD_RUNGS: one rung at most
      if (k < (u32)TD_RUNGS) {
        const u32 s = atomicAdd(&S.n[k], 1u);
        if (s < (u32)TD_LIST_CAP) S.idx[k][s] = (u16)(i0 + j * (int)blockDim.x);
      }
    }
  }
  __syncthreads();
}

// Complete factorization of n >= 1 into F (prime order as found). All lanes call.
// Returns false when a bound was hit (status says which). With hard_left, a composite
// cofactor that would need rho (no prime factor below 2^16, not a square) is not factored:
// it is left in *hard_left (0 otherwise) and F holds the other prime factors; the caller
// finishes with warp_factor_cofactor if it needs the rest.
__device__ inline bool warp_factor(u64 n, WarpFac &F, const u32 *__restrict__ tdp, const u64 *__restrict__ tdi,
                                   u32 *status, u32 lane, volatile u64 *rho_slot,
                                   const volatile int *cancel = nullptr, int my_k = 0,
                                   const HardBoard *board = nullptr, u64 rho_budget = WARP_RHO_STEPS,
                                   bool use_ecm = true, u64 *hard_left = nullptr,
                                   const u16 *td_list = nullptr, u32 td_n = ~0u, u32 td_small = 0) {
  if (hard_left) *hard_left = 0;
  if (lane == 0) { F.k = 0; F.overflow = 0; }
  __syncwarp();
  if (n <= 1) return true;
  const int tz = __ffsll((long long)n) - 1;
  if (tz) { n >>= tz; wf_add(F, 2, tz, lane); }
  u64 cur = n;                 // n with every prime found so far divided out
  bool complete = true;        // every odd prime < 2^16 was tested
  // Blocks of TD_UNROLL chunks of 32 primes, lane i of chunk c testing prime 32c + i: n is
  // divisible by an odd prime d iff x = n * d^-1 (mod 2^64) satisfies x * d < 2^64, i.e.
  // umul64hi(x, d) == 0 (then x = n / d exactly). The table holds only d (tdp) and d^-1 (tdi),
  // 12 bytes a prime, 78 KB in all, small enough to stay in L1; the loads of the next block
  // are issued before the current block is tested, so the loop pays one load latency rather
  // than one per block. Testing primes past the point where d^2 > cur is harmless (each prime
  // is tested once, against n, and a hit is a genuine factor), so the early exit is checked
  // once per block.
  // Divides out of cur every prime of this chunk that divides n (hit: x = n / d exactly), with
  // its full power, and records it in F.
  auto take = [&](bool hit, u64 x, u64 iv, u32 d) {
    const unsigned mask = __ballot_sync(FULL, hit);
    if (!mask) return;                             // rare: a prime below 2^16 divides n
    u64 f = 1;
    int e = 0;
    if (hit) {
      u64 m = x;
      e = 1;
      f = iv;
      for (int g = 0; g < 64; ++g) {
        x = m * iv;
        if (__umul64hi(x, (u64)d)) break;
        m = x; ++e; f *= iv;
      }
    }
    const int base = F.k;
    __syncwarp();
    if (hit) {
      const int pos = base + __popc(mask & ((1u << lane) - 1));
      if (pos < MAXF) { F.pr[pos] = d; F.ex[pos] = e; }
    }
    u64 g = f;
    #pragma unroll
    for (int o = 16; o; o >>= 1) g *= __shfl_xor_sync(FULL, g, o);
    cur *= g;                                      // exact: divides out every d^e found
    __syncwarp();
    if (lane == 0) {
      const int nk = base + __popc(mask);
      if (nk > MAXF) F.overflow = 1;
      F.k = nk > MAXF ? MAXF : nk;
    }
    __syncwarp();
  };
  if (td_list && td_n <= (u32)TD_LIST_CAP) {       // the block's sieve listed n's odd primes < 2^16
    const u32 ns = __popc(td_small);               // lanes [0, ns): the small ones, then the list
    bool mine = false;
    u32 i = 0;
    if (lane < ns) {
      u32 m = td_small;
      for (u32 t = 0; t < lane; ++t) m &= m - 1;
      i = (u32)(__ffs(m) - 1);
      mine = true;
    } else if (lane < ns + td_n) {
      i = (u32)td_list[lane - ns];
      mine = true;
    }
    const u64 iv = mine ? __ldg(tdi + i) : 0;
    const u32 d = mine ? __ldg(tdp + i) : 0u;
    const u64 x = n * iv;
    take(mine && __umul64hi(x, (u64)d) == 0, x, iv, d);
  } else {
  constexpr int TD_UNROLL = 8;
  u64 inv[TD_UNROLL], ninv[TD_UNROLL];
  u32 pr[TD_UNROLL], npr[TD_UNROLL];
  auto load_block = [&](int cb, u64 (&iv)[TD_UNROLL], u32 (&pv)[TD_UNROLL]) {
    #pragma unroll
    for (int j = 0; j < TD_UNROLL; ++j) {
      const int i = (cb + j) * 32 + lane;
      iv[j] = i < NTD ? __ldg(tdi + i) : 0;
      pv[j] = i < NTD ? __ldg(tdp + i) : 0;
    }
  };
  load_block(0, inv, pr);
  for (int cb = 0; cb < TD_CHUNKS; cb += TD_UNROLL) {
    if (cb + TD_UNROLL < TD_CHUNKS) load_block(cb + TD_UNROLL, ninv, npr);
    const int nx = (cb + TD_UNROLL) * 32;
    #pragma unroll
    for (int j = 0; j < TD_UNROLL; ++j) {
      const int i = (cb + j) * 32 + lane;
      const u64 x = n * inv[j];
      take(i < NTD && __umul64hi(x, (u64)pr[j]) == 0, x, inv[j], pr[j]);
    }
    if (nx >= NTD) break;
    const u64 dn = __shfl_sync(FULL, (u64)npr[0], 0);   // the next block's first prime
    if (dn * dn > cur) { complete = false; break; }   // cur is 1 or prime
    if (cancel && __shfl_sync(FULL, cancelled(cancel, my_k) ? 1 : 0, 0)) return false;   // moot rung
    #pragma unroll
    for (int j = 0; j < TD_UNROLL; ++j) { inv[j] = ninv[j]; pr[j] = npr[j]; }
  }
  }
  if (cur > 1) {
    if (!complete || cur <= 0xFFFFFFFFull) {
      wf_add(F, cur, 1, lane);
    } else if (hard_left) {
      const u64 s = isqrt64(cur);
      if (warp_is_prime(cur, lane)) wf_add(F, cur, 1, lane);
      else if (s * s == cur) wf_add(F, s, 2, lane);     // s is prime: no factor of cur is below 2^16
      else *hard_left = cur;                             // needs rho: left to the caller
    } else {
      return warp_factor_cofactor(cur, F, status, lane, rho_slot, cancel, my_k, board, rho_budget, use_ecm);
    }
  }
  __syncwarp();
  if (F.overflow) { if (lane == 0) atomicOr(status, ST_FAC_OVERFLOW); return false; }
  return true;
}

// 128-bit product bound: a*b <= q for a, b < 2^128, q < 2^128 (one of a, b must be below
// 2^64 for the product to fit at all).
__device__ __forceinline__ bool mul_le128(U128 a, U128 b, U128 q, U128 &out) {
  if (a.hi && b.hi) return false;
  if (a.hi) { const U128 t = a; a = b; b = t; }     // now a < 2^64
  bool over;
  out = mul128_64(b, a.lo, over);
  return !over && !lt128(q, out);
}

struct DPWarp {            // shared memory, one per warp: the DP's table and the next one, in turn
  U128 v[2][RCAP + 1];
};

// Residues modulo a rung's r (1 <= r <= RCAP) without a division per residue: Barrett
// reduction of 32-bit values with m = floor((2^32 - 1) / r) (the quotient estimate umulhi(x, m)
// is low by at most one, r = 1 and powers of two included), and 64-bit values from their
// halves with c = 2^32 mod r.
struct ModR {
  u32 r, m, c;
  __device__ __forceinline__ explicit ModR(u32 r_) : r(r_), m(0xFFFFFFFFu / r_) {
    const u32 rem = 0xFFFFFFFFu - m * r_;
    c = rem + 1 == r_ ? 0u : rem + 1;
  }
  __device__ __forceinline__ u32 mod32(u32 x) const {
    const u32 v = x - __umulhi(x, m) * r;
    return v >= r ? v - r : v;
  }
  __device__ __forceinline__ u32 mod64(u64 x) const {
    return mod32(mod32((u32)(x >> 32)) * c + mod32((u32)x));   // below RCAP^2 + RCAP < 2^32
  }
};

// min_div_res (sieve/rung_scan3.cpp:544-565), lanes over residue classes. Returns the
// least divisor u <= q of q^2 with u == target (mod r), or 0.
__device__ inline U128 warp_min_div_res(u64 p, const WarpFac &F, U128 q, u32 r, u32 target, DPWarp &D, u32 lane) {
  const U128 INF{~0ull, ~0ull};
  const ModR R(r);
  const u32 one = r == 1 ? 0u : 1u;              // 1 mod r
  // p's own stage: q = pA with A < p, so p^2 > q and p enters with exponent 0 or 1 -- the
  // divisors 1 and p (this one only when p is within the bound)
  const u32 pm = R.mod64(p);
  const bool p_fits = !lt128(q, U128{p, 0});
  u32 ph = 0;                                     // D.v[ph] is the current table
  for (u32 t = lane; t < r; t += 32)
    D.v[0][t] = (t == one) ? U128{1, 0} : (p_fits && t == pm) ? U128{p, 0} : INF;
  __syncwarp();
  for (int idx = 0; idx < F.k; ++idx) {
    const u64 pr = F.pr[idx];
    const int e = 2 * (int)F.ex[idx];
    const u32 prm = R.mod64(pr);
    u32 inv = 0;                                 // prm^-1 mod r (prm is a unit: gcd(q, r) = 1)
    for (u32 base = 0; base < r; base += 32) {
      const u32 x = base + lane;
      const unsigned m = __ballot_sync(FULL, x < r && R.mod32(prm * x) == one);
      if (m) { inv = base + __ffs(m) - 1; break; }
    }
    for (u32 t = lane; t < r; t += 32) {
      U128 best = INF;
      u32 s = t;
      U128 pw{1, 0};
      for (int j = 0; j <= e; ++j) {
        if (j) {
          bool over;
          pw = mul128_64(pw, pr, over);
          if (over || lt128(q, pw)) break;       // pr^j > q: nothing further fits
          s = R.mod32(s * inv);
        }
        const U128 v = D.v[ph][s];
        if (v.lo == ~0ull && v.hi == ~0ull) continue;
        U128 cand;
        if (mul_le128(v, pw, q, cand) && lt128(cand, best)) best = cand;
      }
      D.v[ph ^ 1][t] = best;
    }
    __syncwarp();                                  // every lane has read D.v[ph]: swap
    ph ^= 1;
  }
  const U128 u = D.v[ph][target];
  __syncwarp();
  return (u.lo == ~0ull && u.hi == ~0ull) ? U128{0, 0} : u;
}

struct RungResult { u64 A; u32 r, k; U128 u; };

// Rung k of p's walk (the loop body of solve_rung3, sieve/rung_scan3.cpp:578-603): r = r0 + 4k
// with r0 the least positive r = -p (mod 4), A = (p + r) / 4, q = pA, and the residue the
// divisor must have, target = -q (mod r). False when the rung does not apply (r > RCAP, A = 0,
// or q not prime to r).
struct Rung { u64 A; U128 q; u32 r, target; };
__device__ __forceinline__ u32 rung_r0(u64 p) { return 4 - (u32)(p & 3); }
__device__ __forceinline__ bool rung_of(u64 p, u32 k, Rung &g) {
  const u32 r = rung_r0(p) + 4 * k;
  if (k > RCAP || r > RCAP) return false;
  const u64 A = (p >> 2) + ((u64)(p & 3) + r) / 4;
  if (!A) return false;
  const ModR R(r);
  const u32 qm = R.mod32(R.mod64(p) * R.mod64(A));
  if (r > 1 && gcd64(qm, r) != 1) return false;
  g = Rung{A, U128{p * A, __umul64hi(p, A)}, r, qm ? r - qm : 0};
  return true;
}

// Below this bound a divisor of q^2 = (pA)^2 cannot involve p or a prime factor of a cofactor
// that trial division left (every such prime is at least 65537, the first prime after the
// trial-division table's last, 65521).
constexpr u64 SMALL_U_BOUND = 65536;
#ifndef ES_SMALL_U
#define ES_SMALL_U 1
#endif

// min_div_res of one rung (sieve/rung_scan3.cpp:544-565): the least divisor u <= q of q^2,
// q = pA, with u == target (mod r), or u = 0 when there is none. A is factored by trial
// division first; when that leaves a composite cofactor C (prime factors all >= 65537), the
// divisors of q^2 below 65537 are exactly those of S^2, S = A / C, so the least qualifying
// one among them -- found from S's primes alone -- is the answer whenever it exists, and C is
// factored (rho, ECM) only when it does not. The same u comes out either way. Returns false
// when a bound was hit or the rung was cancelled.
__device__ inline bool rung_divisor(u64 p, u64 A, U128 q, u32 r, u32 target, WarpFac &F, DPWarp &D,
                                    const u32 *tdp, const u64 *tdi, u32 *status, u32 lane,
                                    volatile u64 *rho_slot, const volatile int *cancel, int my_k,
                                    const HardBoard *board, u64 rho_budget, bool use_ecm, U128 &u,
                                    const u16 *td_list = nullptr, u32 td_n = ~0u, u32 td_small = 0) {
  u64 hard = 0;
  if (!warp_factor(A, F, tdp, tdi, status, lane, rho_slot, cancel, my_k, board, rho_budget, use_ecm,
                   ES_SMALL_U ? &hard : nullptr, td_list, td_n, td_small))
    return false;
  if (hard) {
    u = warp_min_div_res(p, F, U128{SMALL_U_BOUND, 0}, r, target, D, lane);
    if (u.lo || u.hi) return true;
    if (!warp_factor_cofactor(hard, F, status, lane, rho_slot, cancel, my_k, board, rho_budget, use_ecm)) return false;
  }
  u = warp_min_div_res(p, F, q, r, target, D, lane);
  return true;
}

// The rung walk of one prime by one warp, rung after rung (solve_rung3,
// sieve/rung_scan3.cpp:578-603, in its own order): the throughput form of block_solve_rung
// below, for while there are more primes than warps. Returns true in every lane when a rung
// certifies p, with the result in *out (written by lane 0). use_ecm = false keeps the hard
// cofactors on rho: with every warp of the GPU busy, a round of curves costs more issue slots
// than the rho steps it saves (a 10^14-integer window at 10^16, a million primes: 108 ms of
// stage D with rho alone, 179 ms with ECM), while ECM pays in the latency-bound tail.
__device__ inline bool warp_solve_rung(u64 p, const u32 *tdp, const u64 *tdi, u32 *status, WarpFac &F,
                                       DPWarp &D, volatile u64 *rho_slot, RungResult *out,
                                       const HardBoard *board = nullptr, u64 rho_budget = WARP_RHO_STEPS,
                                       bool use_ecm = true) {
  const u32 lane = threadIdx.x & 31;
  const u32 r0 = rung_r0(p);
  for (u32 k = 0; r0 + 4 * k <= RCAP; ++k) {
    Rung g;
    if (!rung_of(p, k, g)) continue;
    U128 u;
    if (!rung_divisor(p, g.A, g.q, g.r, g.target, F, D, tdp, tdi, status, lane, rho_slot, nullptr, 0, board,
                      rho_budget, use_ecm, u))
      return false;
    if (u.lo == 0 && u.hi == 0) continue;
    if (lane == 0) *out = RungResult{g.A, g.r, k, u};
    __syncwarp();
    return true;
  }
  return false;
}

#ifndef ES_TD_SIEVE
#define ES_TD_SIEVE 1
#endif
// The rung walk of one prime by a block of W warps (solve_rung3, sieve/rung_scan3.cpp:
// 578-603). Warp w takes rung indices k = w, w+W, ... (r = r0 + 4k) in increasing order and
// stops once k passes the best certifying index found by any warp. With S the block first
// lists the odd primes below 2^16 of all the prime's rungs at once (block_td_sieve), and each
// rung divides out only its own. Returns true in every thread when some rung certifies p;
// the block's result is then in *out.
template <int W>
__device__ inline bool block_solve_rung(u64 p, const u32 *tdp, const u64 *tdi, const uint2 *tdqm, TdSieve *S,
                                        u32 *status, WarpFac *F, DPWarp *D, volatile u64 *rho_slot, int *best_k,
                                        RungResult *slot, RungResult *out, const HardBoard *board = nullptr,
                                        u64 rho_budget = WARP_RHO_STEPS) {
  const u32 lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  BlockHelp *const bh = board ? board->local : nullptr;
  if (threadIdx.x == 0) {
    *best_k = 0x7FFFFFFF;
    if (bh) { bh->n = 0; bh->found = 0; bh->busy = W; }
  }
  if (lane == 0) slot[w].k = 0x7FFFFFFF;
  __syncthreads();
  if (!ES_TD_SIEVE) S = nullptr;
  if (S) block_td_sieve((p >> 2) + 1, tdqm, *S);   // A_0 = floor(p/4) + 1
  const u32 r0 = rung_r0(p);
  for (u32 k = w; r0 + 4 * k <= RCAP; k += W) {
    // warp-uniform: every lane must take the same branch before the warp collectives below
    if ((int)k >= __shfl_sync(FULL, *(volatile int *)best_k, 0)) break;
    Rung g;
    if (!rung_of(p, k, g)) continue;
    U128 u;
    if (!rung_divisor(p, g.A, g.q, g.r, g.target, F[w], D[w], tdp, tdi, status, lane, rho_slot + w, best_k, (int)k,
                      board, rho_budget, true, u, S ? S->idx[k] : nullptr, S ? S->n[k] : ~0u, S ? S->small[k] : 0u))
      break;
    if (u.lo == 0 && u.hi == 0) continue;
    if (lane == 0) {
      slot[w] = RungResult{g.A, g.r, k, u};
      atomicMin(best_k, (int)k);
    }
    break;
  }
  if (bh) {                                     // done with this prime's rungs: help the others
    if (lane == 0) atomicSub(&bh->busy, 1u);
    __syncwarp();
    if (ES_LOCAL_HELP) warp_help_block(bh, lane);
  }
  __syncthreads();
  const int bk = *(volatile int *)best_k;
  bool ok = false;
  if (bk != 0x7FFFFFFF) {
    ok = true;
    if (threadIdx.x == 0)
      for (int i = 0; i < W; ++i) if ((int)slot[i].k == bk) *out = slot[i];
  }
  __syncthreads();
  return ok;
}

}  // namespace es
