// es_kernels.cuh -- device-side layouts shared by the kernels and the host engine.
#pragma once
#include <cstdint>
#include "es_arith.cuh"

namespace es {

constexpr u16 K0_MISS = 0xFFFF;     // the filter never hits this lane
constexpr int DMAX = 8192;          // distinct strides held in shared memory per CTA

// One scan window as the device sees it. Lane l's positions are p = rho_l + M*K for
// K = Kfirst .. Kfirst + npos - 1, with Kfirst = Q + (rho_l < lo mod M). Segment-marking
// items (k_mark) are (lane, segment) pairs with segments of SEG_BIG positions. Windows with
// at most SEG_SMALL positions per lane (and sub-windows of that size cut from longer ones)
// go to the kill-mask kernel instead; SEG_SMALL is the length of the mask repeat. 128
// measured best over the 4096-window batch and 10^14-integer windows together (64: 2% faster
// on the batch, 20% slower on long windows; 256: 6% slower on the batch).
constexpr u32 GROUP = 16;
#ifndef ES_SEG_SMALL
#define ES_SEG_SMALL 128
#endif
constexpr u32 SEG_SMALL = ES_SEG_SMALL;
constexpr u32 SEG_BIG = 16384;

struct WinDev {
  u64 lo, hi;
  u64 Q;          // lo / M
  u64 item0;      // first marking item of this window in the batch's item space
  u32 lomod;      // lo % M
  u32 G;          // lanes per item (1 or GROUP)
  u32 seg;        // positions per segment
  u32 nseg;       // segments
  u32 lane0;      // first lane of the active range (a multiple of G)
  u32 groups;     // lane groups per segment
};

// Sizes of the batch in flight, read by the marking kernels from device memory so that one
// captured launch sequence (a CUDA graph) serves every batch up to the buffers' capacity.
struct BatchHdr {
  u64 total_items;   // long-window marking items
  u32 nwin, nshort;  // windows; short windows
};

// A position that no filter killed: (window, lane, J) is its key in the output order.
struct Surv {
  u64 p;
  u64 J;
  u32 win, lane;
};

// Per-window device counters; covered/sieved/mr are derived on the host from
// positions, alive-after-covers and survivors, which are sums over segments, and the
// composites from the survivors less the primes (rung + direct + unsolved).
struct WinCount {
  unsigned long long positions, after_covers, surv, spare, rung, direct, unsolved, pad;
};

// Device record: the layout of es_record.
struct RecDev {
  u32 kind, win, lane, reserved;
  u64 J, p, a, b, c, d;
};

struct MarkParams {
  const u32 *rho;          // [L] lane classes
  const u16 *K0;           // [L][ldk] first hit K mod s per (lane, filter), or K0_MISS
  const u32 *fdesc;        // [nf] stride s (low 16 bits) | index of s among distinct strides
  const u32 *sdist;        // [D] distinct strides
  const u16 *Qm;           // [nwin][Dq] (lo / M) mod s_d per window (rows of Dq >= D, 16-byte multiples)
  const WinDev *win;       // [nwin]
  u64 *queue;              // work-queue head (persistent schedule)
  Surv *surv;              // survivor list
  unsigned long long *surv_count;
  WinCount *cnt;           // [nwin]
  const BatchHdr *hdr;     // total_items, nwin
  u64 surv_cap;
  u64 M;
  u32 L, ldk, nf, ncov, D, Dq;
  u32 r_bytes;             // shared bytes for the stride residues (16-aligned)
};

// Short windows (at most SEG_SMALL positions in any lane) are marked from per-(lane, stride)
// kill masks: for lane l and a stride s shared by several filters, bit x of the mask is set
// when some filter of that stride kills K == x (mod s); bits [s, s + SEG_SMALL) repeat the
// pattern so that the positions of a whole segment starting below s are consecutive bits,
// read 32 at a time as funnel shifts of consecutive words.
constexpr u32 MASK_BYTES_MAX = 48 * 1024;   // per-lane mask table budget (shared memory)

// One masked stride: s, its index in sdist, the 32-bit word offset of its slice in a lane's
// table, and the log2 of the distance between the slice's consecutive words. The strides of
// the first INTERLEAVE_ROUNDS rounds of 32 (the densest, which every short window walks) are
// stored interleaved -- word w of the stride in slot 32g + j at off = base_g + j, w at
// off + 32 w, sh = 5 -- so that lane j of a warp reading any word of its own stride reads
// shared-memory bank j; the other strides are packed one after another (sh = 0).
struct MaskDesc { u32 s, d, off, sh; };
#ifndef ES_INTERLEAVE_ROUNDS
#define ES_INTERLEAVE_ROUNDS 2
#endif
constexpr u32 INTERLEAVE_ROUNDS = ES_INTERLEAVE_ROUNDS;

// A short window as k_mark_short walks it: lanes outside [la, lb) have no position in it.
// Lane rho holds lq + [(rho - lo) mod M < lr] positions, lq = len / M, lr = len mod M (the
// count of p == rho (mod M) in [lo, lo + len)).
struct ShortWin {
  u64 Q;
  u32 lomod, wi, la, lb, lq, lr;
};

struct ShortParams {
  const u32 *rho;
  const u16 *K0;
  const u32 *fdesc;
  const u16 *Qm;            // [nwin][Dq]
  const u64 *mtab;          // [L][Wpad] kill masks
  const MaskDesc *mdesc;    // covers' mask strides [0, nm_cov), then stage B' [nm_cov, nm_all)
  const u32 *lfil;          // filters not covered by a mask: covers [0, nl_cov), then B' [nl_cov, nl_all)
  const WinDev *win;
  const ShortWin *shortw;   // the short windows
  Surv *surv;
  unsigned long long *surv_count;
  WinCount *cnt;
  u64 surv_cap, M;
  const BatchHdr *hdr;      // nshort
  u32 L, ldk, D, Dq, Wpad, nm_cov, nm_all, nl_cov, nl_all;
};

struct HardSlot;

struct TailParams {
  Surv *surv;
  unsigned long long *surv_count;
  u32 *cand;               // indices into surv that passed the base-2 round
  unsigned long long *cand_count;
  u32 *primes;             // indices into surv
  unsigned long long *prime_count;
  u32 *direct;             // indices into surv, primes that no rung certified
  unsigned long long *direct_count;
  RecDev *recs;
  unsigned long long *rec_count;
  WinCount *cnt;
  const u32 *tdp;          // odd primes < 2^16
  const TdEntry *tde;      // their inverses mod 2^64 and division limits (thread-per-value paths)
  const u64 *tdi;          // their inverses mod 2^64 alone (warp trial division)
  const uint2 *tdqm;       // {d, floor(2^32 / d)} (the rung sieve's residues)
  u32 *status;
  u64 cap;                 // capacity of surv/primes/direct/recs
  unsigned long long *rung_next;      // k_rung's prime queue head, whole blocks (the tail)
  unsigned long long *rung_next_warp; // k_rung's prime queue head, one warp per prime
  unsigned long long *rung_done;      // primes k_rung has finished
  unsigned long long *help_sessions;  // helping sessions started on the hard board
  struct HardSlot *board;             // [HARD_SLOTS] cofactors whose rho takes long
  u32 help_blocks;                    // k_rung blocks [0, help_blocks) help on the board
  u64 rho_budget;                     // Brent steps per lane before a factorization gives up
};

}  // namespace es
