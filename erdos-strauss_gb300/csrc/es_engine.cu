// es_engine.cu -- the GB300 engine: device tables, the funnel kernels, and the C ABI.
//
// Data layout in HBM (resident for the engine's lifetime):
//   rho[L]            u32  lane classes mod M in wheel order
//   K0[L][ldk]        u16  per (lane, filter): the residue K0 = K mod s at which filter f
//                          kills lane l (p = rho_l + M*K), or K0_MISS; 2308 x 3752 x 2 B
//                          = 17.3 MB for the M = 2042040 table, read coalesced row by row
//   mtab[L][Wpad]     u64  per lane, one kill mask per distinct stride s: bit x set when some
//                          filter of stride s kills K = x (mod s), for x < s + SEG_SMALL
//                          (33.4 KB a lane, 77 MB for the M = 2042040 table)
//   mdesc             per masked stride (densest first): s, its Qm column, its mask offset
//   fdesc[nf]         u32  per filter: stride s = mod/gcd(M,mod) and its Qm column
//   tdp/tde                trial-division table: 6541 odd primes < 2^16 with inverses
// Per run: window and short-window descriptors, Qm[window][stride] = (lo / M) mod s, the
// survivor list, prime/direct index lists, records, counters and the hard board.
//
// Pipeline per run (one CUDA stream, replayed as a CUDA graph for batches):
//   k_prep        Qm for every window and stride
//   k_mark_short  a CTA per pair of lanes with their mask rows in shared memory; each warp
//                 walks short windows (and 128-position pieces of long ones): rounds of 32
//                 strides, one funnel-shift extraction of 32 positions per stride and chunk,
//                 a warp OR, stopping when every position is dead; survivors appended
//   k_mark        the alternative for long windows: a byte map per segment in shared memory,
//                 each filter clears its progression, warp-aggregated compaction
//   k_mr          a thread per survivor: the base-2 strong-probable-prime round
//   k_mr2         a warp per number that passed base 2: the 12-base test, one base per lane
//   k_rung        stage D: a warp per prime while primes outnumber the grid's warps, then a
//                 block of four warps per prime over successive rungs; warp trial division,
//                 Miller-Rabin, Brent's rho, ECM rounds (es_tail.cuh, es_ecm.cuh), the rung
//                 DP, and the exact certificate check (es_check.cuh) before a record is
//                 written
//   k_direct      a thread per prime left over: the direct search, else SURVIVOR
// Records come back unordered; the host puts them in (window, lane, J) order, the
// reference's lane-major order per window.
#include "../../include/es_sieve.h"
#include "es_arith.cuh"
#include "es_check.cuh"
#include "es_kernels.cuh"
#include "es_tail.cuh"
#include "es_wheel.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <type_traits>
#include <chrono>
#include <cinttypes>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

namespace es {

// ============================================================================ kernels

// K0 table: for lane l and filter f, p = rho + M*K == res (mod mod) iff
// g | (res - rho) and K == ((res - rho) mod mod)/g * inv((M/g) mod s, s) (mod s).
// This is the per-(lane, filter) setup of sieve/rung_scan3.cpp:719-728 moved from the
// window's first position to K = 0, so it no longer depends on the window at all.
__global__ void k_build_k0(const u32 *__restrict__ rho, u32 L, const u64 *__restrict__ mods,
                           const u64 *__restrict__ ress, const u32 *__restrict__ gs,
                           const u32 *__restrict__ invs, const u32 *__restrict__ fdesc, u32 nf,
                           u32 ldk, u16 *__restrict__ K0) {
  const u64 idx = (u64)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (u64)L * ldk) return;
  const u32 l = (u32)(idx / ldk), f = (u32)(idx % ldk);
  if (f >= nf) { K0[idx] = K0_MISS; return; }
  const u64 mod = mods[f];
  const u64 d = (ress[f] % mod + mod - rho[l] % mod) % mod;
  const u32 g = gs[f], s = fdesc[f] & 0xFFFFu;
  if (d % g) { K0[idx] = K0_MISS; return; }
  K0[idx] = (u16)((d / g) * (u64)invs[f] % s);
}


// Clear the progression of every filter in [from, to) over alive[0, n) of one lane.
template <int BLOCK>
__device__ __forceinline__ void mark_lane(const u16 *__restrict__ K0row, const u32 *__restrict__ fdesc,
                                          const u16 *R, unsigned char *alive, u32 from, u32 to, u32 n) {
  for (u32 f = from + threadIdx.x; f < to; f += BLOCK) {
    const u32 k0 = K0row[f];
    if (k0 == K0_MISS) continue;
    const u32 fd = __ldg(fdesc + f);
    const u32 s = fd & 0xFFFFu;
    int off = (int)k0 - (int)R[fd >> 16];
    if (off < 0) off += (int)s;
    for (u32 j = (u32)off; j < n; j += s) alive[j] = 0;
  }
}

template <int BLOCK>
__device__ __forceinline__ u32 block_sum(u32 v, u32 *red) {
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
  const int wid = threadIdx.x >> 5, ln = threadIdx.x & 31;
  __syncthreads();
  if (ln == 0) red[wid] = v;
  __syncthreads();
  u32 t = 0;
  if (threadIdx.x < 32) {
    t = threadIdx.x < BLOCK / 32 ? red[threadIdx.x] : 0;
    for (int o = 16; o; o >>= 1) t += __shfl_xor_sync(0xFFFFFFFFu, t, o);
  }
  return t;   // valid in thread 0
}

struct ItemInfo {
  u64 J0;                 // position index of the segment start within each lane
  u64 first[GROUP];       // first position p of each lane in the window
  u32 n[GROUP];           // positions of each lane in this segment (0 = inactive)
  u32 lane_base, win, G, bmask, valid;
};

// Per-window residues (lo / M) mod s_d for every distinct stride: computed once per window
// here, instead of once per (window, lane) item.
// Qm[w][d] = Q_w mod s_d. A thread keeps its strides d = threadIdx.x + k blockDim over the
// block's windows, with the Barrett constant of each stride taken once: Q < 2^64 / M, so Q mod
// s for s < 2^16 is three 16-bit steps of a 32-bit reduction (the quotient estimate
// umulhi(x, m), m = floor((2^32 - 1) / s), is low by at most one).
__global__ void k_prep(const BatchHdr *__restrict__ hdr, const WinDev *__restrict__ win,
                       const u32 *__restrict__ sdist, u32 D, u32 Dq, u16 *__restrict__ Qm) {
  const u32 nwin = hdr->nwin;
  for (u32 d = threadIdx.x; d < D; d += blockDim.x) {
    const u32 sd = sdist[d], m = 0xFFFFFFFFu / sd;
    auto mod = [&](u32 x) { const u32 v = x - __umulhi(x, m) * sd; return v >= sd ? v - sd : v; };
    for (u32 w = blockIdx.x; w < nwin; w += gridDim.x) {
      const u64 Q = win[w].Q;
      u32 r = mod((u32)(Q >> 32));
      r = mod((r << 16) | ((u32)(Q >> 16) & 0xFFFFu));
      r = mod((r << 16) | ((u32)Q & 0xFFFFu));
      Qm[(size_t)w * Dq + d] = (u16)r;
    }
  }
}

// Items are dealt from an atomic queue (persistent schedule: gridDim = resident CTAs) or
// one per CTA (gridDim = items).
template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) k_mark(const MarkParams P, int persistent) {
  extern __shared__ __align__(16) unsigned char smem[];
  u16 *R0 = reinterpret_cast<u16 *>(smem);          // G = 1: R; G = GROUP: residues at K = Q
  u16 *R1 = R0 + P.D;                                // G = GROUP: residues at K = Q + 1
  unsigned char *alive = smem + P.r_bytes;
  u32 *alive32 = reinterpret_cast<u32 *>(alive);
  __shared__ ItemInfo it;
  __shared__ u32 red[BLOCK / 32];
  __shared__ u64 s_item;
  const u32 lane_id = threadIdx.x & 31;
  const u64 total_items = P.hdr->total_items;
  const u32 nwin = P.hdr->nwin;
  u64 next = blockIdx.x;
  for (;;) {
    if (threadIdx.x == 0) {
      const u64 item = persistent ? atomicAdd(reinterpret_cast<unsigned long long *>(P.queue), 1ull) : next;
      s_item = item;
      it.valid = 0;
      if (item < total_items) {
        u32 lo = 0, hi = nwin;                     // last window with item0 <= item
        while (hi - lo > 1) {
          const u32 mid = (lo + hi) >> 1;
          if (P.win[mid].item0 <= item) lo = mid; else hi = mid;
        }
        const WinDev &W = P.win[lo];
        const u64 rem = item - W.item0;
        it.win = lo;
        it.G = W.G;
        it.lane_base = W.lane0 + (u32)(rem % W.groups) * W.G;
        it.J0 = (rem / W.groups) * W.seg;
        it.valid = 1;
      }
    }
    __syncthreads();
    const u64 item = s_item;
    if (item >= total_items) break;
    next += gridDim.x;
    const u32 win = it.win, G = it.G, lane_base = it.lane_base;
    const u64 J0 = it.J0;
    const WinDev &W = P.win[win];
    if (threadIdx.x < G) {
      const u32 lane = lane_base + threadIdx.x;
      u32 n = 0;
      u64 first = 0;
      bool b = false;
      if (lane < P.L) {
        const u64 rho = P.rho[lane];
        b = rho < W.lomod;
        const u64 Kfirst = W.Q + (b ? 1 : 0);
        first = rho + P.M * Kfirst;
        if (first < W.hi) {
          const u64 npos = (W.hi - first - 1) / P.M + 1;
          if (J0 < npos) n = (u32)min((u64)W.seg, npos - J0);
        }
      }
      it.n[threadIdx.x] = n;
      it.first[threadIdx.x] = first;
      const unsigned bm = __ballot_sync(0xFFFFFFFFu >> (32 - (G < 32 ? G : 32)), b);
      if (threadIdx.x == 0) it.bmask = bm;
    }
    __syncthreads();
    u32 ntot = 0;
    #pragma unroll
    for (int g = 0; g < (int)GROUP; ++g) ntot += (g < (int)G) ? it.n[g] : 0;
    if (ntot == 0) { __syncthreads(); continue; }
    // segment-start residues of K modulo every distinct stride
    const u16 *Qm = P.Qm + (size_t)win * P.Dq;
    if (G == 1) {
      const u32 b = it.bmask & 1;
      for (u32 d = threadIdx.x; d < P.D; d += BLOCK) {
        const u32 s = P.sdist[d];
        u32 r = (u32)Qm[d] + b + (J0 ? (u32)(J0 % s) : 0u);
        r = r >= s ? r - s : r;
        r = r >= s ? r - s : r;
        R0[d] = (u16)r;
      }
    } else {
      for (u32 d = threadIdx.x; d < P.D; d += BLOCK) {
        const u32 s = P.sdist[d], q = Qm[d];
        R0[d] = (u16)q;
        R1[d] = (u16)(q + 1 == s ? 0 : q + 1);
      }
    }
    // alive bytes: 1 for the segment's positions, 0 beyond
    const u32 nw = G == 1 ? (it.n[0] + 3) >> 2 : GROUP * (SEG_SMALL / 4);
    for (u32 w = threadIdx.x; w < nw; w += BLOCK) {
      const u32 g = G == 1 ? 0 : w / (SEG_SMALL / 4);
      const u32 jb = (G == 1 ? w : w % (SEG_SMALL / 4)) * 4;
      const u32 n = it.n[g];
      const u32 left = n > jb ? n - jb : 0;
      alive32[w] = left >= 4 ? 0x01010101u : (0x01010101u & ((1u << (8 * left)) - 1u));
    }
    __syncthreads();
    u32 ng[GROUP];
    #pragma unroll
    for (int g = 0; g < (int)GROUP; ++g) ng[g] = (g < (int)G) ? it.n[g] : 0;
    for (int phase = 0; phase < 2; ++phase) {
      const u32 from = phase ? P.ncov : 0, to = phase ? P.nf : P.ncov;
      if (phase) {                                  // stage B': count survivors of the covers
        if (P.nf == P.ncov) break;
        u32 c = 0;
        for (u32 w = threadIdx.x; w < nw; w += BLOCK) c += __popc(alive32[w]);
        c = block_sum<BLOCK>(c, red);
        if (threadIdx.x == 0) atomicAdd(&P.cnt[win].after_covers, (unsigned long long)c);
      }
      mark_lane<BLOCK>(P.K0 + (size_t)lane_base * P.ldk, P.fdesc, R0, alive, from, to, ng[0]);   // G == 1
      __syncthreads();
    }
    // Compaction: each warp takes 32 consecutive words per step; an inclusive warp scan of
    // the per-word popcounts gives each lane its slot, and one atomicAdd per warp reserves
    // the warp's block in the survivor list.
    u32 mine = 0;
    const u32 wid = threadIdx.x >> 5;
    for (u32 base = wid * 32; base < nw; base += BLOCK) {
      const u32 w = base + lane_id;
      u32 x = w < nw ? alive32[w] : 0u;
      const u32 c = __popc(x);
      u32 incl = c;
      #pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const u32 t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane_id >= (u32)o) incl += t;
      }
      const u32 tot = __shfl_sync(0xFFFFFFFFu, incl, 31);
      if (tot) {
        unsigned long long gbase = 0;
        if (lane_id == 0) gbase = atomicAdd(P.surv_count, (unsigned long long)tot);
        gbase = __shfl_sync(0xFFFFFFFFu, gbase, 0);
        u64 slot = gbase + incl - c;
        const u32 g = G == 1 ? 0 : w / (SEG_SMALL / 4);
        const u32 jb = (G == 1 ? w : w % (SEG_SMALL / 4)) * 4;
        while (x) {
          const u32 k = __ffs(x) - 1;
          x &= x - 1;
          if (slot < P.surv_cap) {
            const u64 J = J0 + jb + (k >> 3);
            Surv sv;
            sv.p = it.first[g] + P.M * J;
            sv.J = J;
            sv.win = win;
            sv.lane = lane_base + g;
            P.surv[slot] = sv;
          }
          ++slot;
        }
        mine += tot;
      }
    }
    if (lane_id == 0 && mine) atomicAdd(&P.cnt[win].surv, (unsigned long long)mine);
    __syncthreads();
  }
}

// ---------------------------------------------------------------- short windows
// A CTA holds the kill-mask tables of SHORT_LANES consecutive lanes in shared memory; each
// warp takes one short window at a time and marks the segments of those lanes in it. The
// per-window work that does not depend on the lane -- the stride descriptor and the
// segment-start residue (lo / M) mod s -- is done once for all SHORT_LANES lanes.
#ifndef ES_SHORT_LANES
#define ES_SHORT_LANES 2
#endif
constexpr int SHORT_LANES = ES_SHORT_LANES;
// Windows with at most SPARSE_N positions in either lane of a k_mark_short CTA take the sparse
// first round (short_sparse_round). Measured on the 4096-window batch: 0.87 ms for the kernel
// with 32, 0.98 without the sparse round, 0.88 with 16, 0.93 with 48 or 64 (a second chunk
// per lane: the task path marks those windows for less).
#ifndef ES_SPARSE_N
#define ES_SPARSE_N 32
#endif
constexpr u32 SPARSE_N = ES_SPARSE_N;
static_assert(SPARSE_N <= 32, "a sparse window's positions fit one 32-position chunk per lane");
constexpr u32 HAND_WORDS = SHORT_LANES;          // alive words per window handed on, one per lane
constexpr u32 SMD_MAX = 512;       // stride descriptors staged in shared memory


__device__ __forceinline__ u32 warp_or32(u32 v) { return __reduce_or_sync(0xFFFFFFFFu, v); }

// Mask strides [m0, m1) over the segments of SHORT_LANES lanes, in rounds of 32 strides (one
// per lane of the warp). alive[q][c] holds the positions 32c + j of lane q's segment not yet
// killed; it is the same in every lane of the warp. A segment starts at K == Qrow[d] + b[q]
// (mod s_d); mask bits come out 32 at a time: word r/32 + c and the next, funnel-shifted right
// by r mod 32. After each round the warp ORs its kill words into alive, and it stops as soon
// as nothing is left alive: the strides come densest first, so most segments are dead after
// one or two rounds. Returns nonzero if a position is still alive.

#ifndef ES_FIRST_SH
#define ES_FIRST_SH 1
#endif
template <int NC>
__device__ __forceinline__ u32 short_mask_rounds(u32 (&alive)[SHORT_LANES][NC], const u32 (&b)[SHORT_LANES],
                                                 const u32 *tab, u32 tab_words, const MaskDesc *smd, u32 m0,
                                                 u32 m1, const u16 *__restrict__ Qrow, u32 q0_first, u32 lane,
                                                 const MaskDesc &md_first) {
  u32 kill[SHORT_LANES][NC];
  // Round one (strides m0 .. m0 + 31, q0_first loaded by the caller ahead of time): every
  // chunk, one mask word load per chunk, no per-chunk tests.
  u32 k = m0 + lane;
  u32 q0 = k + 32 < m1 ? (u32)__ldg(Qrow + smd[k + 32].d) : 0u;    // the next round's residue
  if (k < m1) {
    const MaskDesc md = md_first;                    // this lane's stride of the first round
    // SH: the round's row layout (the same for all its strides), a constant in each copy
    auto first = [&](auto shc) {
      constexpr u32 SH = decltype(shc)::value;
      u32 r = 0;
      #pragma unroll
      for (int q = 0; q < SHORT_LANES; ++q) {
        if (q == 0 || b[q] != b[0]) {                // lanes whose segments start together share r
          r = q0_first + b[q];
          r = r >= md.s ? r - md.s : r;
        }
        // the mask repeats for SEG_SMALL bits past s, so chunk c is words r/32 + c, + c + 1
        const u32 *wp = tab + q * tab_words + md.off + ((r >> 5) << (SH == 1 ? md.sh : SH));
        const u32 sh = r & 31;
        u32 w0 = wp[0];
        #pragma unroll
        for (int c = 0; c < NC; ++c) {
          const u32 w1 = wp[(c + 1) << (SH == 1 ? md.sh : SH)];
          kill[q][c] = __funnelshift_r(w0, w1, sh);
          w0 = w1;
        }
      }
    };
    if (!ES_FIRST_SH) first(std::integral_constant<u32, 1>{});   // 1: the layout read at run time
    else if (md.sh == 5) first(std::integral_constant<u32, 5>{});
    else first(std::integral_constant<u32, 0>{});
  } else {
    #pragma unroll
    for (int q = 0; q < SHORT_LANES; ++q)
      #pragma unroll
      for (int c = 0; c < NC; ++c) kill[q][c] = 0;
  }
  u32 any = 0;
  #pragma unroll
  for (int q = 0; q < SHORT_LANES; ++q)
    #pragma unroll
    for (int c = 0; c < NC; ++c) {
      alive[q][c] &= ~warp_or32(kill[q][c]);
      any |= alive[q][c];
    }
  // Later rounds, rarely more than one or two: only the chunks still alive.
  for (u32 kb = m0 + 32; kb < m1 && any; kb += 32) {
    k = kb + lane;
    const u32 q0_next = k + 32 < m1 ? (u32)__ldg(Qrow + smd[k + 32].d) : 0u;
    #pragma unroll
    for (int q = 0; q < SHORT_LANES; ++q)
      #pragma unroll
      for (int c = 0; c < NC; ++c) kill[q][c] = 0;
    if (k < m1) {
      const MaskDesc md = smd[k];
      #pragma unroll
      for (int q = 0; q < SHORT_LANES; ++q) {
        u32 r = q0 + b[q];
        r = r >= md.s ? r - md.s : r;
        const u32 *wp = tab + q * tab_words + md.off + ((r >> 5) << md.sh);
        const u32 sh = r & 31;
        #pragma unroll
        for (int c = 0; c < NC; ++c)
          if (alive[q][c]) kill[q][c] = __funnelshift_r(wp[c << md.sh], wp[(c + 1) << md.sh], sh);
      }
    }
    q0 = q0_next;
    any = 0;
    #pragma unroll
    for (int q = 0; q < SHORT_LANES; ++q)
      #pragma unroll
      for (int c = 0; c < NC; ++c)
        if (alive[q][c]) {
          alive[q][c] &= ~warp_or32(kill[q][c]);
          any |= alive[q][c];
        }
  }
  return any;
}

// kill[q][c] gets bit j set when position 32c + j of lane q's segment is hit by one of the
// filters lfil[l0, l1) (the strides without a mask), checked one by one from the first-hit
// table. Lanes of the warp split the filters; the caller reduces.
template <int NC>
__device__ __forceinline__ void short_list_kill(u32 (&kill)[SHORT_LANES][NC], const u32 (&n)[SHORT_LANES],
                                                const u32 (&b)[SHORT_LANES], const u32 *__restrict__ lfil, u32 l0,
                                                u32 l1, const u16 *const (&K0row)[SHORT_LANES],
                                                const u32 *__restrict__ fdesc, const u16 *__restrict__ Qrow,
                                                u32 lane) {
  for (u32 k = l0 + lane; k < l1; k += 32) {
    const u32 f = lfil[k];
    const u32 fd = __ldg(fdesc + f);
    const u32 s = fd & 0xFFFFu;
    const u32 q0 = (u32)__ldg(Qrow + (fd >> 16));
    #pragma unroll
    for (int q = 0; q < SHORT_LANES; ++q) {
      const u32 k0 = K0row[q][f];
      if (k0 == K0_MISS) continue;
      u32 r = q0 + b[q];
      r = r >= s ? r - s : r;
      int off = (int)k0 - (int)r;
      if (off < 0) off += (int)s;
      for (u32 j = (u32)off; j < n[q]; j += s) {
        #pragma unroll
        for (int c = 0; c < NC; ++c)
          if ((j >> 5) == (u32)c) kill[q][c] |= 1u << (j & 31);
      }
    }
  }
}

// One phase (covers, or the stage-B' primes) over alive: the mask strides [m0, m1), then, if
// anything survived them, the unmasked filters lfil[l0, l1). Returns the positions alive.
template <int NC>
__device__ __forceinline__ u32 short_phase(u32 (&alive)[SHORT_LANES][NC], const ShortParams &P, const u32 *tab,
                                           u32 tab_words, const MaskDesc *smd, u32 m0, u32 m1, u32 l0, u32 l1,
                                           const u32 (&n)[SHORT_LANES], const u32 (&b)[SHORT_LANES],
                                           const u16 *const (&K0row)[SHORT_LANES], const u16 *Qrow, u32 q0_first,
                                           u32 lane, const MaskDesc &md_first) {
  const u32 any = short_mask_rounds<NC>(alive, b, tab, tab_words, smd, m0, m1, Qrow, q0_first, lane, md_first);
  if (any && l1 > l0) {
    u32 kill[SHORT_LANES][NC];
    #pragma unroll
    for (int q = 0; q < SHORT_LANES; ++q)
      #pragma unroll
      for (int c = 0; c < NC; ++c) kill[q][c] = 0;
    short_list_kill<NC>(kill, n, b, P.lfil, l0, l1, K0row, P.fdesc, Qrow, lane);
    #pragma unroll
    for (int q = 0; q < SHORT_LANES; ++q)
      #pragma unroll
      for (int c = 0; c < NC; ++c) alive[q][c] &= ~warp_or32(kill[q][c]);
  }
  u32 cnt = 0;
  #pragma unroll
  for (int q = 0; q < SHORT_LANES; ++q)
    #pragma unroll
    for (int c = 0; c < NC; ++c) cnt += __popc(alive[q][c]);
  return cnt;
}


// The segments of SHORT_LANES lanes in one short window, NC 32-position chunks each.
// The window a warp is marking: its index, and the lane of the warp holding its descriptor
// (whose q_lo/q_hi registers carry Q = lo / M, read only when there are survivors).
struct WinRef {
  u32 wi, q_lo, q_hi;
  int src;
};

template <int NC>
__device__ __forceinline__ void short_segments(const ShortParams &P, const u32 *tab, u32 tab_words,
                                               const MaskDesc *smd, u32 l_first, const WinRef &R,
                                               const u64 (&rho)[SHORT_LANES], const u32 (&n)[SHORT_LANES],
                                               const u32 (&b)[SHORT_LANES], const u16 *const (&K0row)[SHORT_LANES],
                                               u32 q0_first, u32 lane, const MaskDesc &md0, const u32 *hand_j) {
  const u32 wi = R.wi;
  const u16 *Qrow = P.Qm + (size_t)wi * P.Dq;
  u32 alive[SHORT_LANES][NC];
  u32 cnt;
  if (NC == 1 && hand_j) {                         // the sparse round did the first round
    #pragma unroll
    for (int q = 0; q < SHORT_LANES; ++q) alive[q][0] = hand_j[q];
    const u32 k = 32 + lane;
    const MaskDesc md1 = k < P.nm_cov ? smd[k] : MaskDesc{1, 0, 0, 0};
    const u32 q1 = k < P.nm_cov ? (u32)__ldg(Qrow + md1.d) : 0u;
    cnt = short_phase<NC>(alive, P, tab, tab_words, smd, min(32u, P.nm_cov), P.nm_cov, 0, P.nl_cov, n, b, K0row,
                          Qrow, q1, lane, md1);
  } else {
    #pragma unroll
    for (int q = 0; q < SHORT_LANES; ++q)
      #pragma unroll
      for (int c = 0; c < NC; ++c) {
        const u32 lo = 32 * c;
        alive[q][c] = n[q] >= lo + 32 ? ~0u : (n[q] > lo ? (1u << (n[q] - lo)) - 1 : 0u);
      }
    cnt = short_phase<NC>(alive, P, tab, tab_words, smd, 0, P.nm_cov, 0, P.nl_cov, n, b, K0row, Qrow, q0_first,
                          lane, md0);
  }
  if (cnt && (P.nm_all > P.nm_cov || P.nl_all > P.nl_cov)) {          // stage B'
    if (lane == 0) atomicAdd(&P.cnt[wi].after_covers, (unsigned long long)cnt);
    const u32 k = P.nm_cov + lane;
    const u32 q0b = k < P.nm_all ? (u32)__ldg(Qrow + smd[k].d) : 0u;
    const MaskDesc mdb = k < P.nm_all ? smd[k] : MaskDesc{1, 0, 0, 0};
    cnt = short_phase<NC>(alive, P, tab, tab_words, smd, P.nm_cov, P.nm_all, P.nl_cov, P.nl_all, n, b, K0row, Qrow,
                          q0b, lane, mdb);
  }
  if (!cnt) return;
  // survivors are rare: the window's first position index comes from its lane, and lane 0
  // writes the survivors in order
  const u64 Q = (u64)__shfl_sync(FULL, R.q_lo, R.src) | ((u64)__shfl_sync(FULL, R.q_hi, R.src) << 32);
  if (lane == 0) {
    u64 slot = atomicAdd(P.surv_count, (unsigned long long)cnt);
    atomicAdd(&P.cnt[wi].surv, (unsigned long long)cnt);
    #pragma unroll
    for (int q = 0; q < SHORT_LANES; ++q)
      #pragma unroll
      for (int c = 0; c < NC; ++c) {
        u32 x = alive[q][c];
        while (x) {
          const u32 k = __ffs(x) - 1;
          x &= x - 1;
          if (slot < P.surv_cap) {
            const u64 J = 32 * c + k;
            Surv sv;
            sv.p = rho[q] + P.M * (Q + b[q] + J);        // the segment starts at K = Q + b
            sv.J = J;
            sv.win = wi;
            sv.lane = l_first + q;
            P.surv[slot] = sv;
          }
          ++slot;
        }
      }
  }
}

// The sparse windows of a 32-window group (at most SPARSE_N positions in either lane of the
// CTA: windows shorter than a few wheel periods) get the first round of strides alone, window
// after window with the next window's residue loaded ahead: lane k extracts the kill word of
// stride k for both lanes' positions, one warp OR each, and nothing else -- no task set-up.
// The first round kills all but ~1% of positions, so almost every sparse window ends there;
// the few with a position still alive are returned as a mask of the group's lanes, their alive
// words left in hand[window][lane], and the task path goes on with them from the second round.
// Counters and survivors are the task path's alone.

// SH is the first round's row layout, the same for every stride of the round: 5 when its rows
// are interleaved (word w of the stride in slot j at 32 w + j), 0 when they are packed.
template <u32 SH>
__device__ __forceinline__ unsigned short_sparse_round(const ShortParams &P, const u32 *tab, u32 tab_words,
                                                       const MaskDesc &md0, u32 xwi, u32 pk, unsigned sp,
                                                       u32 *hand, u32 lane) {
  static_assert(SHORT_LANES == 2, "two lanes per CTA");
  const bool has = lane < P.nm_cov;                // lane k holds the first round's stride k
  auto ldq = [&](u32 wi) { return has ? (u32)__ldg(P.Qm + (size_t)wi * P.Dq + md0.d) : 0u; };
  unsigned again = 0;
  // this lane's own window of the group: its positions in the CTA's two lanes as bit masks
  // (at most SPARSE_N each when the window is sparse)
  const u32 n0l = pk & 255u, n1l = (pk >> 8) & 255u;
  const u32 lm0 = n0l >= 32 ? ~0u : (1u << n0l) - 1, lm1 = n1l >= 32 ? ~0u : (1u << n1l) - 1;
  u32 qn = ldq(__shfl_sync(FULL, xwi, __ffs(sp) - 1));
  while (sp) {
    const int j = __ffs(sp) - 1;
    sp &= sp - 1;
    const u32 pj = __shfl_sync(FULL, pk, j);
    const u32 m0 = __shfl_sync(FULL, lm0, j), m1 = __shfl_sync(FULL, lm1, j);
    const u32 qd = qn;
    if (sp) qn = ldq(__shfl_sync(FULL, xwi, __ffs(sp) - 1));
    u32 kill0 = 0, kill1 = 0;
    if (has) {
      u32 r = qd + ((pj >> 24) & 1u);
      r = r >= md0.s ? r - md0.s : r;
      const u32 *wp = tab + md0.off + ((r >> 5) << SH);
      kill0 = __funnelshift_r(wp[0], wp[1u << SH], r & 31);
      if ((pj ^ (pj >> 1)) & (1u << 24)) {       // the two lanes' segments start apart (rare)
        r = qd + ((pj >> 25) & 1u);
        r = r >= md0.s ? r - md0.s : r;
      }
      wp = tab + tab_words + md0.off + ((r >> 5) << SH);
      kill1 = __funnelshift_r(wp[0], wp[1u << SH], r & 31);
    }
    const u32 a0 = m0 & ~warp_or32(kill0);
    const u32 a1 = m1 & ~warp_or32(kill1);
    if (a0 | a1) {                                  // the task path goes on from the second round
      again |= 1u << j;
      if (lane == 0) { hand[j * HAND_WORDS] = a0; hand[j * HAND_WORDS + 1] = a1; }
    }
  }
  __syncwarp();
  return again;
}

template <int BLOCK>
__global__ void __launch_bounds__(BLOCK, 2) k_mark_short(const ShortParams P) {
  extern __shared__ __align__(16) u32 tab[];
  const u32 lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (P.hdr->nshort == 0) return;
  const u32 tab_words = P.Wpad * 2;                    // 32-bit words per lane table
  // the stride descriptors (at most SMD_MAX, the host keeps any further strides unmasked)
  MaskDesc *smd = reinterpret_cast<MaskDesc *>(tab + SHORT_LANES * tab_words);
  for (u32 k = threadIdx.x; k < P.nm_all; k += BLOCK) smd[k] = P.mdesc[k];
  u32 *hand = reinterpret_cast<u32 *>(smd + P.nm_all) + warp * 32 * HAND_WORDS;   // this warp's hand-on
  const u32 nshort = P.hdr->nshort;
  for (u32 l0 = blockIdx.x * SHORT_LANES; l0 < P.L; l0 += gridDim.x * SHORT_LANES) {
    for (int q = 0; q < SHORT_LANES; ++q) {
      const u32 l = min(l0 + q, P.L - 1);              // a missing last lane loads a copy; it stays inactive
      const uint4 *src = reinterpret_cast<const uint4 *>(P.mtab + (size_t)l * P.Wpad);
      uint4 *dst = reinterpret_cast<uint4 *>(tab + q * tab_words);
      for (u32 i = threadIdx.x; i < P.Wpad / 2; i += BLOCK) dst[i] = __ldg(src + i);
    }
    __syncthreads();
    u64 rho[SHORT_LANES];
    const u16 *K0row[SHORT_LANES];
    #pragma unroll
    for (int q = 0; q < SHORT_LANES; ++q) {
      const u32 l = min(l0 + q, P.L - 1);
      rho[q] = P.rho[l];
      K0row[q] = P.K0 + (size_t)l * P.ldk;
    }
    // This warp's windows are i = warp + WS t. They are read 32 at a time, one descriptor per
    // lane in one load, and each lane works out the segments of this CTA's lanes in its window
    // (positions n and start offset b); a ballot keeps the windows where either lane has a
    // position and the warp walks those, taking n and b packed in one shuffle. The first
    // round's stride residue of the next window is loaded while a window is marked.
    constexpr u32 WS = BLOCK / 32;
    const uint4 *sw4 = reinterpret_cast<const uint4 *>(P.shortw);
    const MaskDesc md0 = lane < P.nm_cov ? smd[lane] : MaskDesc{1, 0, 0, 0};   // the first round's stride
    const u32 sh0 = P.nm_cov ? smd[0].sh : 0u;          // its layout (the same for the round's strides)
    const u32 d_first = md0.d;
    auto load_q0 = [&](u32 wi) {
      return lane < P.nm_cov ? (u32)__ldg(P.Qm + (size_t)wi * P.Dq + d_first) : 0u;
    };
    static_assert(SHORT_LANES <= 3 && SEG_SMALL < 256, "n (8 bits) and b of each lane are packed in one word");
    for (u32 t0 = 0; warp + WS * t0 < nshort; t0 += 32) {
      const u32 my = warp + WS * (t0 + lane);
      uint4 x = make_uint4(0, 0, 0, 0), y = make_uint4(0, 0, 0, 0);
      if (my < nshort) { x = __ldg(sw4 + 2 * (size_t)my); y = __ldg(sw4 + 2 * (size_t)my + 1); }
      // fields: x = {Q lo, Q hi, lomod, wi}, y = {la, lb, lq, lr}
      u32 pk = 0;                                  // n_q at bit 8q, b_q at bit 24 + q
      if (my < nshort) {
        #pragma unroll
        for (int q = 0; q < SHORT_LANES; ++q) {
          const u32 l = l0 + q;
          const u32 r = (u32)rho[q];
          const u32 bq = r < x.z ? 1u : 0u;
          const u32 d = r + (bq ? (u32)P.M : 0u) - x.z;              // (rho - lo) mod M
          const u32 nq = (l < P.L && l >= y.x && l < y.y) ? y.z + (d < y.w ? 1u : 0u) : 0u;
          pk |= (nq << (8 * q)) | (bq << (24 + q));
        }
      }
      u32 nmax_w = 0;
      #pragma unroll
      for (int q = 0; q < SHORT_LANES; ++q) nmax_w = max(nmax_w, (pk >> (8 * q)) & 255u);
      unsigned todo = __ballot_sync(FULL, nmax_w > SPARSE_N);
      unsigned hand_mask = 0;                      // windows the sparse round handed on
      if (SPARSE_N) {
        const unsigned sp = __ballot_sync(FULL, nmax_w > 0 && nmax_w <= SPARSE_N);
        if (sp) hand_mask = sh0 ? short_sparse_round<5>(P, tab, tab_words, md0, x.w, pk, sp, hand, lane)
                                : short_sparse_round<0>(P, tab, tab_words, md0, x.w, pk, sp, hand, lane);
        todo |= hand_mask;
      }
      u32 q0n = todo ? load_q0(__shfl_sync(FULL, x.w, __ffs(todo) - 1)) : 0u;
      while (todo) {
        const int j = __ffs(todo) - 1;
        todo &= todo - 1;
        const u32 pj = __shfl_sync(FULL, pk, j);
        const u32 wi = __shfl_sync(FULL, x.w, j);
        const u32 q0_first = q0n;
        if (todo) q0n = load_q0(__shfl_sync(FULL, x.w, __ffs(todo) - 1));
        u32 n[SHORT_LANES], b[SHORT_LANES], nmax = 0;
        #pragma unroll
        for (int q = 0; q < SHORT_LANES; ++q) {
          n[q] = (pj >> (8 * q)) & 255u;
          b[q] = (pj >> (24 + q)) & 1u;
          nmax = max(nmax, n[q]);
        }
        const WinRef R{wi, x.x, x.y, j};
        const u32 *hj = (hand_mask >> j) & 1u ? hand + j * HAND_WORDS : nullptr;
        // chunks per lane; one chunk is by far the commonest case, so it is tested first.
        const u32 nc = (nmax + 31) >> 5;
        // instantiations for 1, 2 and 4 chunks (8 too when SEG_SMALL is 256) measured faster
        // than one per chunk count: the kernel's code stays small enough for the instruction
        // cache
        if (nc == 1) short_segments<1>(P, tab, tab_words, smd, l0, R, rho, n, b, K0row, q0_first, lane, md0, hj);
        else if (nc == 2) short_segments<2>(P, tab, tab_words, smd, l0, R, rho, n, b, K0row, q0_first, lane, md0, hj);
        else if constexpr (SEG_SMALL > 128) {
          if (nc <= 4) short_segments<4>(P, tab, tab_words, smd, l0, R, rho, n, b, K0row, q0_first, lane, md0, hj);
          else short_segments<8>(P, tab, tab_words, smd, l0, R, rho, n, b, K0row, q0_first, lane, md0, hj);
        } else if constexpr (SEG_SMALL > 64) {
          short_segments<4>(P, tab, tab_words, smd, l0, R, rho, n, b, K0row, q0_first, lane, md0, hj);
        }
      }
    }
    __syncthreads();
  }
}

// Kill masks from the first-hit table: bit x of lane l's mask for filter f's stride, for
// every x == K0[l][f] (mod s) below s + SEG_SMALL (the repeat that a segment of up to
// SEG_SMALL positions starting below s may reach).
__global__ void k_build_masks(const u16 *__restrict__ K0, u32 L, u32 ldk, u32 nf, const int *__restrict__ fmask,
                              const MaskDesc *__restrict__ mdesc, u32 Wpad, u64 *__restrict__ mtab) {
  const u64 idx = (u64)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (u64)L * nf) return;
  const u32 l = (u32)(idx / nf), f = (u32)(idx % nf);
  const int m = fmask[f];
  if (m < 0) return;
  const u32 k0 = K0[(size_t)l * ldk + f];
  if (k0 == K0_MISS) return;
  const MaskDesc md = mdesc[m];
  u32 *row = reinterpret_cast<u32 *>(mtab + (size_t)l * Wpad) + md.off;
  for (u32 x = k0; x < md.s + SEG_SMALL; x += md.s) atomicOr(row + ((x >> 5) << md.sh), 1u << (x & 31));
}

// Miller-Rabin in two passes. Nearly every survivor is composite and fails the base-2
// round (sprp2, sieve/rung_scan3.cpp:680-689), so pass one runs that round with a thread per
// survivor; the few that pass get the 12-base test (census/rung_scan.cpp:76-92) with one base
// per lane of a warp. A prime passes base 2, so the two passes give exactly is_prime.
__global__ void k_mr(const TailParams T) {
  const u64 n = min((u64)*T.surv_count, T.cap);
  for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x) {
    const Surv s = T.surv[i];
    if (sprp2_64(s.p)) {
      const unsigned long long k = atomicAdd(T.cand_count, 1ull);
      if (k < T.cap) T.cand[k] = (u32)i;
    }
  }
}

__global__ void k_mr2(const TailParams T) {
  const u32 lane = threadIdx.x & 31;
  const u64 warps = (u64)gridDim.x * blockDim.x / 32;
  const u64 n = min((u64)*T.cand_count, T.cap);
  for (u64 i = ((u64)blockIdx.x * blockDim.x + threadIdx.x) / 32; i < n; i += warps) {
    const u32 si = T.cand[i];
    const Surv s = T.surv[si];
    const bool prime = warp_is_prime(s.p, lane);
    if (lane == 0) {
      if (prime) {
        const unsigned long long k = atomicAdd(T.prime_count, 1ull);
        if (k < T.cap) T.primes[k] = si;
      }
    }
  }
}

__device__ __forceinline__ void put_record(const TailParams &T, const RecDev &r) {
  const unsigned long long k = atomicAdd(T.rec_count, 1ull);
  if (k < T.cap) T.recs[k] = r;
}

#ifndef ES_RUNG_WARPS
#define ES_RUNG_WARPS 4
#endif
constexpr int RUNG_WARPS = ES_RUNG_WARPS;
#ifndef ES_RUNG_TAIL_PER_BLOCK
#define ES_RUNG_TAIL_PER_BLOCK RUNG_WARPS     // primes per block left for the block phase
#endif
#ifndef ES_RUNG_MIN_BLOCKS
#define ES_RUNG_MIN_BLOCKS (16 / RUNG_WARPS)   // resident blocks per SM the register budget allows
#endif
#ifndef ES_HELP_BLOCKS_PER_SM
#define ES_HELP_BLOCKS_PER_SM 1
#endif
#ifndef ES_FEW_ECM_DIV
#define ES_FEW_ECM_DIV 4
#endif
#ifndef ES_FEW_ECM_AFTER
#define ES_FEW_ECM_AFTER 384
#endif
#ifndef ES_HELP_FEW_DIV
#define ES_HELP_FEW_DIV 16
#endif
#ifndef ES_HELP_BLOCKS_DIV
#define ES_HELP_BLOCKS_DIV 1
#endif

// Stage D. While more primes remain than the grid has warps, every warp takes a prime of its
// own from a queue and walks its rungs in order (warp_solve_rung: no barrier, no speculative
// rungs); the last gridDim.x * RUNG_WARPS primes go to whole blocks of RUNG_WARPS warps that
// try four rungs of one prime at a time (block_solve_rung), so that the run ends on short
// latencies. A block that finds both queues empty turns its warps into helpers on the hard
// board (warp_help) until every prime of the run is finished, so that the last, hardest
// factorizations get more walks than one warp's.
__device__ __forceinline__ void rung_result(const TailParams &T, const Surv &s, u32 si, bool ok,
                                            const RungResult &res) {
  if (ok && !check_rung_cert(s.p, res.A, res.r, res.u)) {
    atomicOr(T.status, ST_CERT_BAD);                // never emitted
  } else if (ok) {
    RecDev rec{ES_REC_RUNG, s.win, s.lane, 0, s.J, s.p, res.A, res.r, res.u.lo, res.u.hi};
    put_record(T, rec);
    atomicAdd(&T.cnt[s.win].rung, 1ull);
  } else {
    const unsigned long long k = atomicAdd(T.direct_count, 1ull);
    if (k < T.cap) T.direct[k] = si;
  }
  __threadfence();
  atomicAdd(T.rung_done, 1ull);
}

__global__ void __launch_bounds__(RUNG_WARPS * 32, ES_RUNG_MIN_BLOCKS) k_rung(const TailParams T, int no_rung) {
  __shared__ WarpFac F[RUNG_WARPS];
  __shared__ DPWarp D[RUNG_WARPS];
  __shared__ u64 rho_slot[RUNG_WARPS];
  __shared__ int best_k;
  __shared__ RungResult slot[RUNG_WARPS];
  __shared__ RungResult res;
  __shared__ unsigned long long next;
  const u64 n = min((u64)*T.prime_count, T.cap);
  const u32 lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __shared__ BlockHelp bhelp;
  __shared__ TdSieve tds;
  HardBoard B;
  B.slot = T.board; B.sessions = T.help_sessions; B.done = T.rung_done; B.total = n;
  B.local = nullptr;                                 // the warp phase: no block-mates on one prime
  // A run of few primes is bound by the latency of its hardest factorizations, on SMs that are
  // otherwise idle: its cofactors turn to curves sooner.
  B.ecm_after = (ES_FEW_ECM_DIV && n * ES_FEW_ECM_DIV <= (u64)gridDim.x) ? ES_FEW_ECM_AFTER : 0;
  const u64 tail = min(n, (u64)gridDim.x * ES_RUNG_TAIL_PER_BLOCK);
  const u64 nw = n - tail;                           // primes [0, nw): a warp each
  for (;;) {
    u64 i = 0;
    if (lane == 0) i = atomicAdd(T.rung_next_warp, 1ull);
    i = __shfl_sync(0xFFFFFFFFu, i, 0);
    if (i >= nw) break;
    const u32 si = T.primes[i];
    const Surv s = T.surv[si];
    const bool ok = !no_rung && warp_solve_rung(s.p, T.tdp, T.tdi, T.status, F[w], D[w], rho_slot + w, &slot[w], &B,
                                                T.rho_budget, /*use_ecm=*/false);
    if (lane == 0) rung_result(T, s, si, ok, slot[w]);
    __syncwarp();
  }
  __syncthreads();
  B.local = &bhelp;
  for (;;) {                                          // primes [nw, n): a block each
    if (threadIdx.x == 0) next = nw + atomicAdd(T.rung_next, 1ull);
    __syncthreads();
    const u64 i = next;
    if (i >= n) break;
    const u32 si = T.primes[i];
    const Surv s = T.surv[si];
    const bool ok = !no_rung &&
                    block_solve_rung<RUNG_WARPS>(s.p, T.tdp, T.tdi, T.tdqm, &tds, T.status, F, D, rho_slot, &best_k, slot,
                                                 &res, &B,
                                                 T.rho_budget);
    if (threadIdx.x == 0) rung_result(T, s, si, ok, res);
    __syncthreads();
  }
  // Helpers come from the first help_blocks blocks only (one per SM): the walks of a hard
  // cofactor progress at the issue rate their sub-partition gives them, so helpers beyond
  // one warp per scheduler would only split that rate over more walks, and the expected wait
  // for the first collision grows with the square root of the number of walks sharing it.
  // They help only a run of few primes (at most one per ES_HELP_FEW_DIV blocks), whose time
  // is its slowest factorization on SMs that are otherwise idle: the 2^34 window at 1.8e19
  // with the tuned table (21 primes) 0.33 against 0.46 ms of stage D. With more primes the
  // helpers' walks take issue slots from the owners (129 primes: 0.375 against 0.36 ms;
  // batches: 0.48 against 0.435 ms before this rule), and a pipelined tail would keep its
  // blocks resident.
  B.local = nullptr;
  const bool few = ES_HELP_FEW_DIV == 0 || n * ES_HELP_FEW_DIV <= (u64)gridDim.x;
  if (!no_rung && few && blockIdx.x < T.help_blocks) warp_help(B, lane);
}

__global__ void k_direct(const TailParams T) {
  const u64 n = min((u64)*T.direct_count, T.cap);
  for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x) {
    const Surv s = T.surv[T.direct[i]];
    u64 a, c, d, k;
    if (solve_direct(s.p, a, c, d, k, T.tdp, T.tde, T.status)) {
      if (!check_solved_cert(s.p, a, c, d, k)) { atomicOr(T.status, ST_CERT_BAD); continue; }
      RecDev rec{ES_REC_SOLVED, s.win, s.lane, 0, s.J, s.p, a, c, d, k};
      put_record(T, rec);
      atomicAdd(&T.cnt[s.win].direct, 1ull);
    } else {
      RecDev rec{ES_REC_SURVIVOR, s.win, s.lane, 0, s.J, s.p, 0, 0, 0, 0};
      put_record(T, rec);
      atomicAdd(&T.cnt[s.win].unsolved, 1ull);
    }
  }
}

// ---------------------------------------------------------------- probe kernels
// Exact re-check of caller records (es_check_records): ok[i] = 1 for a RUNG or SOLVED
// record whose identity holds, 0 otherwise (SURVIVOR and unknown kinds included).
__global__ void k_probe_check(const RecDev *r, u64 count, unsigned char *ok) {
  for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (u64)gridDim.x * blockDim.x) {
    const RecDev x = r[i];
    bool good = false;
    if (x.kind == ES_REC_RUNG) good = check_rung_cert(x.p, x.a, x.b, U128{x.c, x.d});
    else if (x.kind == ES_REC_SOLVED) good = check_solved_cert(x.p, x.a, x.b, x.c, x.d);
    ok[i] = good;
  }
}

__global__ void k_probe_prime(const u64 *n, u64 count, unsigned char *out) {
  const u32 lane = threadIdx.x & 31;
  const u64 warps = (u64)gridDim.x * blockDim.x / 32;
  for (u64 i = ((u64)blockIdx.x * blockDim.x + threadIdx.x) / 32; i < count; i += warps) {
    const bool pr = warp_is_prime(n[i], lane);
    if (lane == 0) out[i] = pr ? 1 : 0;
  }
}
__global__ void __launch_bounds__(RUNG_WARPS * 32, ES_RUNG_MIN_BLOCKS) k_probe_rung(const u64 *p, u64 count, RecDev *out,
                                                               unsigned char *found, const u32 *tdp,
                                                               const u64 *tdi, const uint2 *tdqm, u32 *status,
                                                               u64 rho_budget) {
  __shared__ TdSieve tds;
  __shared__ WarpFac F[RUNG_WARPS];
  __shared__ DPWarp D[RUNG_WARPS];
  __shared__ u64 rho_slot[RUNG_WARPS];
  __shared__ int best_k;
  __shared__ RungResult slot[RUNG_WARPS];
  __shared__ RungResult res;
  for (u64 i = blockIdx.x; i < count; i += gridDim.x) {
    bool ok = block_solve_rung<RUNG_WARPS>(p[i], tdp, tdi, tdqm, &tds, status, F, D, rho_slot, &best_k, slot, &res,
                                           nullptr, rho_budget);
    if (threadIdx.x == 0) {
      if (ok && !check_rung_cert(p[i], res.A, res.r, res.u)) { atomicOr(status, ST_CERT_BAD); ok = false; }
      found[i] = ok;
      out[i] = ok ? RecDev{ES_REC_RUNG, 0, 0, 0, 0, p[i], res.A, res.r, res.u.lo, res.u.hi}
                  : RecDev{0, 0, 0, 0, 0, p[i], 0, 0, 0, 0};
    }
    __syncthreads();
  }
}
__global__ void k_probe_direct(const u64 *p, u64 count, RecDev *out, unsigned char *found,
                               const u32 *tdp, const TdEntry *tde, u32 *status) {
  for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (u64)gridDim.x * blockDim.x) {
    u64 a, c, d, k;
    bool ok = solve_direct(p[i], a, c, d, k, tdp, tde, status);
    if (ok && !check_solved_cert(p[i], a, c, d, k)) { atomicOr(status, ST_CERT_BAD); ok = false; }
    found[i] = ok;
    out[i] = ok ? RecDev{ES_REC_SOLVED, 0, 0, 0, 0, p[i], a, c, d, k} : RecDev{0, 0, 0, 0, 0, p[i], 0, 0, 0, 0};
  }
}
// The production factorization (warp_factor), one warp per value; primes sorted ascending.
__global__ void k_probe_factor(const u64 *n, u64 count, u64 *pr, unsigned char *ex, unsigned char *k,
                               const u32 *tdp, const u64 *tdi, u32 *status, u64 rho_budget) {
  __shared__ WarpFac F[4];
  __shared__ u64 rho_slot[4];
  const u32 lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const u64 warps = (u64)gridDim.x * blockDim.x / 32;
  for (u64 i = ((u64)blockIdx.x * blockDim.x + threadIdx.x) / 32; i < count; i += warps) {
    WarpFac &f = F[w];
    const bool ok = warp_factor(n[i], f, tdp, tdi, status, lane, rho_slot + w, nullptr, 0, nullptr, rho_budget);
    if (lane == 0) {
      const int kk = ok ? f.k : 0;
      for (int a = 1; a < kk; ++a)
        for (int b = a; b > 0 && f.pr[b - 1] > f.pr[b]; --b) {
          const u64 t = f.pr[b]; f.pr[b] = f.pr[b - 1]; f.pr[b - 1] = t;
          const u32 e = f.ex[b]; f.ex[b] = f.ex[b - 1]; f.ex[b - 1] = e;
        }
      for (int a = 0; a < MAXF; ++a) {
        pr[i * MAXF + a] = a < kk ? f.pr[a] : 0;
        ex[i * MAXF + a] = a < kk ? (unsigned char)f.ex[a] : 0;
      }
      k[i] = (unsigned char)kk;
    }
    __syncwarp();
  }
}

// ============================================================================ host engine

constexpr int MARK_BLOCK = 128;
#ifndef ES_SHORT_BLOCK
#define ES_SHORT_BLOCK 512
#endif
constexpr int SHORT_BLOCK = ES_SHORT_BLOCK;
constexpr size_t SHORT_HAND_BYTES = (size_t)(SHORT_BLOCK / 32) * 32 * HAND_WORDS * sizeof(u32);   // 16 warps, 64 registers: two CTAs of two 37 KB lane tables fill an SM

}  // namespace es

namespace es {
// Everything one run needs besides the resident tables: a stream, its events, the per-run
// device buffers and their pinned host staging, and the captured graph. An engine has one
// slot for its synchronous calls and SERVE_SLOTS more for the serving workers, so that
// several batches can be in flight on their own streams.
struct Slot {
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[12] = {};
  BatchHdr *d_hdr = nullptr, *h_hdr = nullptr;
  WinDev *h_win = nullptr;
  ShortWin *h_short = nullptr;
  WinCount *h_cnt = nullptr;
  unsigned long long *h_ctr = nullptr;
  u32 *h_status = nullptr;
  RecDev *h_recs = nullptr;
  // The persistent schedule, captured once per capacity as two graphs: the front (counters
  // cleared, staging copied in, marking, Miller-Rabin) and the tail (stage D, stage E,
  // counters and the record prefix copied out). ev[11] is recorded between them on the
  // slot's stream: the next slot's front waits for it (marking runs one batch at a time, in
  // launch order) while this slot's tail overlaps the next batch's marking.
  cudaGraph_t graph = nullptr, graph2 = nullptr;
  cudaGraphExec_t gexec = nullptr, gexec2 = nullptr;
  WinDev *d_win = nullptr; size_t win_cap = 0;
  WinCount *d_cnt = nullptr;
  ShortWin *d_shortw = nullptr; size_t shortw_cap = 0;
  u16 *d_Qm = nullptr; size_t qm_cap = 0;
  Surv *d_surv = nullptr;
  u32 *d_primes = nullptr, *d_direct = nullptr, *d_cand = nullptr;
  RecDev *d_recs = nullptr;
  size_t cap = 0;
  size_t rec_prefix = 0;                // records the captured graph copies back itself
  unsigned long long *d_ctr = nullptr;  // [0] queue [1] surv [2] prime [3] direct [4] rec [5] cand
                                      // [6] rung queue (blocks) [7] rungs done [8] help sessions
                                      // [9] rung queue (warps), board at [16]
  u32 *d_status = nullptr;
  es_timing_t timing{};
  struct HostScratch {                  // per-run host vectors, kept with their capacity
    std::vector<WinDev> wd;
    std::vector<ShortWin> shortw;
    std::vector<u64> npos;
    std::vector<RecDev> hr;
    std::vector<u32> start, pos;
    std::vector<uint8_t> mag;
    std::vector<es_window> dw;          // the long-window split (run_windows)
    std::vector<std::pair<u32, u64>> dmap;
    std::vector<es_counters> pc;
    std::vector<es_record> all;
  } hs;
  std::mutex mu;                        // one run at a time per slot
};

constexpr int SERVE_SLOTS = 2;
// run counters (16 words) followed by the hard board, cleared together before every run
constexpr size_t CTR_BYTES = 16 * sizeof(unsigned long long) + HARD_SLOTS * sizeof(HardSlot);

// A serving request: windows in, counters and records out.
struct Request {
  uint64_t ticket = 0;
  std::vector<es_window> w;
  std::vector<es_counters> cnt;
  std::vector<es_record> recs;
  es_status st = ES_OK;
  std::string err;
  bool done = false;
  bool claimed = false;                 // an es_poll is waiting on it (one poller per ticket)
  bool solo = false;                    // es_submit_batch: runs as a batch of its own
  u64 mem = 0;                          // admitted device-memory estimate
};
}  // namespace es

struct es_engine {
  // configuration and derived tables
  es::u64 M = 0, mmax = 0, sieve_p = 0;
  uint32_t flags = 0;
  std::vector<es::u64> classes;
  // host arithmetic on window bounds: classes below residue x are lane_at[x >> LANE_BLOCK_BITS]
  // plus the few classes of x's block that lie below x; inv_M estimates division by M
  std::vector<uint32_t> lane_at;
  double inv_M = 0;
  es::u64 wheel_pmin = 0, cover_pmax = 0, class_fnv = 0, filter_fnv = 0;
  const es::ClassPin *pin = nullptr;
  std::vector<es::u64> mods, ress;     // certified filters [0,ncov) then stage-B' primes
  size_t ncov = 0;
  // marking order: filters sorted by stride within each phase
  std::vector<uint32_t> order;
  uint32_t nf = 0, ldk = 0, D = 0, Dq = 0;
  es_schedule sched{es::SEG_SMALL, 6, 1, {0, 0, 0, 0, 0}};   // es_set_schedule / es_autotune
  es::u64 rho_budget = es::WARP_RHO_STEPS;                      // ES_FLAG_TEST_RHO_BUDGET: 64
  int device = 0, sm_count = 0, mark_occupancy = 0;
  // resident device tables
  es::u32 *d_rho = nullptr, *d_fdesc = nullptr, *d_sdist = nullptr, *d_tdp = nullptr;
  es::u16 *d_K0 = nullptr;
  // short-window kill masks
  es::u64 *d_mtab = nullptr;
  es::MaskDesc *d_mdesc = nullptr;
  es::u32 *d_lfil = nullptr;
  uint32_t Wpad = 0, nm_cov = 0, nm_all = 0, nl_cov = 0, nl_all = 0, m_inter = 0;
  es::TdEntry *d_tde = nullptr;
  es::u64 *d_tdi = nullptr;
  uint2 *d_tdqm = nullptr;              // {d, floor(2^32 / d)} for the same primes
  // slot 0: es_run_window / es_run_batch / probes; slots 1..SERVE_SLOTS: serving workers
  es::Slot slots[1 + es::SERVE_SLOTS];
  std::string last_error;
  std::mutex err_mu;
  // serving
  size_t mem_budget = 0;
  std::mutex qmu;
  std::condition_variable qcv, dcv;
  std::deque<es::Request *> queue;
  std::map<uint64_t, es::Request *> reqs;
  uint64_t next_ticket = 1;
  es::u64 mem_in_use = 0;
  size_t queued_windows = 0;
  int pollers = 0;                      // es_poll calls inside the engine (es_close waits for them)
  std::vector<std::thread> workers;
  bool stopping = false;
  // persistent runs of every slot: the slot whose front graph was launched last (its ev[11]
  // marks the end of that front), so that fronts run one after another in launch order
  std::mutex front_mu;
  es::Slot *last_front = nullptr;
};

namespace es {

static es_status fail(es_engine *e, es_status s, const std::string &msg) {
  if (e) { std::lock_guard<std::mutex> lk(e->err_mu); e->last_error = msg; }
  return s;
}

#define CU(call)                                                                           \
  do {                                                                                     \
    cudaError_t err_ = (call);                                                             \
    if (err_ != cudaSuccess)                                                               \
      return fail(e, ES_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(err_));   \
  } while (0)

static void drop_graph(Slot *sl) {
  if (sl->gexec) cudaGraphExecDestroy(sl->gexec);
  if (sl->graph) cudaGraphDestroy(sl->graph);
  if (sl->gexec2) cudaGraphExecDestroy(sl->gexec2);
  if (sl->graph2) cudaGraphDestroy(sl->graph2);
  sl->gexec = sl->gexec2 = nullptr;
  sl->graph = sl->graph2 = nullptr;
}

// Device buffers for nwin windows and a survivor capacity of cap, with their pinned host
// staging. Growing any of them invalidates the captured graph (its copies and kernel
// parameters name the old buffers and sizes).
static es_status ensure_capacity(es_engine *e, Slot *sl, size_t nwin, size_t cap) {
  if (!sl->d_hdr) {
    CU(cudaMalloc(&sl->d_hdr, sizeof(BatchHdr)));
    CU(cudaMallocHost(&sl->h_hdr, sizeof(BatchHdr)));
    CU(cudaMallocHost(&sl->h_ctr, 8 * sizeof(unsigned long long)));
    CU(cudaMallocHost(&sl->h_status, sizeof(u32)));
  }
  if (nwin > sl->win_cap) {
    drop_graph(sl);
    cudaFree(sl->d_win); cudaFree(sl->d_cnt); cudaFree(sl->d_shortw); cudaFree(sl->d_Qm);
    cudaFreeHost(sl->h_win); cudaFreeHost(sl->h_short); cudaFreeHost(sl->h_cnt);
    sl->d_win = nullptr; sl->d_cnt = nullptr; sl->d_shortw = nullptr; sl->d_Qm = nullptr;
    sl->h_win = nullptr; sl->h_short = nullptr; sl->h_cnt = nullptr;
    const size_t want = std::max<size_t>(nwin, 64);
    CU(cudaMalloc(&sl->d_win, want * sizeof(WinDev)));
    CU(cudaMalloc(&sl->d_cnt, want * sizeof(WinCount)));
    CU(cudaMalloc(&sl->d_shortw, want * sizeof(ShortWin)));
    CU(cudaMalloc(&sl->d_Qm, want * std::max<u32>(e->Dq, 8) * sizeof(u16)));
    CU(cudaMallocHost(&sl->h_win, want * sizeof(WinDev)));
    CU(cudaMallocHost(&sl->h_short, want * sizeof(ShortWin)));
    CU(cudaMallocHost(&sl->h_cnt, want * sizeof(WinCount)));
    sl->win_cap = sl->shortw_cap = want;
    sl->qm_cap = want * std::max<u32>(e->Dq, 8);
  }
  if (cap > sl->cap) {
    drop_graph(sl);
    cudaFree(sl->d_surv); cudaFree(sl->d_primes); cudaFree(sl->d_direct); cudaFree(sl->d_recs); cudaFree(sl->d_cand);
    cudaFreeHost(sl->h_recs);
    sl->d_surv = nullptr; sl->d_primes = sl->d_direct = sl->d_cand = nullptr; sl->d_recs = nullptr; sl->h_recs = nullptr;
    CU(cudaMalloc(&sl->d_surv, cap * sizeof(Surv)));
    CU(cudaMalloc(&sl->d_primes, cap * sizeof(u32)));
    CU(cudaMalloc(&sl->d_direct, cap * sizeof(u32)));
    CU(cudaMalloc(&sl->d_cand, cap * sizeof(u32)));
    CU(cudaMalloc(&sl->d_recs, cap * sizeof(RecDev)));
    CU(cudaMallocHost(&sl->h_recs, cap * sizeof(RecDev)));
    sl->cap = cap;
  }
  return ES_OK;
}

static MarkParams mark_params(const es_engine *e, const Slot *sl) {
  MarkParams P;
  P.rho = e->d_rho; P.K0 = e->d_K0; P.fdesc = e->d_fdesc; P.sdist = e->d_sdist;
  P.Qm = sl->d_Qm;
  P.win = sl->d_win; P.queue = reinterpret_cast<u64 *>(sl->d_ctr + 0);
  P.surv = sl->d_surv; P.surv_count = sl->d_ctr + 1; P.cnt = sl->d_cnt;
  P.hdr = sl->d_hdr; P.surv_cap = sl->cap; P.M = e->M;
  P.L = (u32)e->classes.size(); P.ldk = e->ldk; P.nf = e->nf; P.ncov = (u32)e->ncov;
  P.D = e->D; P.Dq = e->Dq;
  P.r_bytes = (4 * e->D + 15) & ~15u;
  return P;
}

// k_mr's grid: a base-2 round is one thread's dependent chain of Montgomery squarings, so
// the launch wants every warp slot the registers allow (40 registers: 8 blocks of 256 per SM);
// measured on the 4096-window batch, 2, 4 and 8 blocks per SM gave 1.346, 1.331 and 1.319 ms
// per step.
#ifndef ES_MR_BLOCKS_PER_SM
#define ES_MR_BLOCKS_PER_SM 8
#endif

static TailParams tail_params(const es_engine *e, const Slot *sl) {
  TailParams T;
  T.surv = sl->d_surv; T.surv_count = sl->d_ctr + 1;
  T.cand = sl->d_cand; T.cand_count = sl->d_ctr + 5;
  T.primes = sl->d_primes; T.prime_count = sl->d_ctr + 2;
  T.direct = sl->d_direct; T.direct_count = sl->d_ctr + 3;
  T.recs = sl->d_recs; T.rec_count = sl->d_ctr + 4;
  T.rung_next = sl->d_ctr + 6; T.rung_done = sl->d_ctr + 7; T.help_sessions = sl->d_ctr + 8;
  T.rung_next_warp = sl->d_ctr + 9;
  T.board = reinterpret_cast<HardSlot *>(sl->d_ctr + 16);
  T.help_blocks = (u32)(e->sm_count * ES_HELP_BLOCKS_PER_SM / ES_HELP_BLOCKS_DIV);
  T.rho_budget = e->rho_budget;
  T.cnt = sl->d_cnt; T.tdp = e->d_tdp; T.tde = e->d_tde; T.tdi = e->d_tdi; T.tdqm = e->d_tdqm; T.status = sl->d_status;
  T.cap = sl->cap;
  return T;
}

static size_t short_smem(const es_engine *e) {
  return (size_t)SHORT_LANES * e->Wpad * 8 + (size_t)e->nm_all * sizeof(MaskDesc) + SHORT_HAND_BYTES;
}

static size_t mark_smem(const es_engine *e) {
  return ((4 * e->D + 15) & ~15u) + std::max<u32>(SEG_BIG, GROUP * SEG_SMALL) + 16;
}

constexpr int LANE_BLOCK_BITS = 9;

// Number of classes below x, 0 <= x <= M (lower_bound over the sorted classes, by table).
static u64 classes_below(const es_engine *e, u64 x) {
  u64 i = e->lane_at[x >> LANE_BLOCK_BITS];
  while (i < e->classes.size() && e->classes[i] < x) ++i;
  return i;
}

// x / M and x mod M for any 64-bit x: a double estimate of the quotient (off by at most
// one: x / M < 2^44, and the product's relative error is 2^-52) corrected exactly.
static void divmod_M(const es_engine *e, u64 x, u64 &q, u64 &r) {
  const u64 M = e->M;
  q = (u64)((double)x * e->inv_M);
  const unsigned __int128 qm = (unsigned __int128)q * M;
  if (qm > x) { --q; r = x - (u64)(qm - M); }
  else { r = x - (u64)qm; if (r >= M) { ++q; r -= M; } }
}

static void build_lane_index(es_engine *e) {
  const u64 nb = (e->M >> LANE_BLOCK_BITS) + 2;
  e->lane_at.assign(nb, 0);
  size_t i = 0;
  for (u64 b = 0; b < nb; ++b) {
    while (i < e->classes.size() && e->classes[i] < (b << LANE_BLOCK_BITS)) ++i;
    e->lane_at[b] = (uint32_t)i;
  }
  e->inv_M = 1.0 / (double)e->M;
}

// Window descriptors and their marking items. Short windows (at most SEG_SMALL positions
// per lane) go to k_mark_short, which walks them lane by lane; long windows get one lane per
// item and segments of SEG_BIG positions in k_mark.
static u64 describe(const es_engine *e, const es_window *w, size_t n, std::vector<WinDev> &out,
                    std::vector<ShortWin> &shortw) {
  out.resize(n);
  shortw.clear();
  shortw.reserve(n);
  u64 items = 0;
  const u64 L = e->classes.size(), M = e->M;
  for (size_t i = 0; i < n; ++i) {
    WinDev &d = out[i];
    d.lo = w[i].lo; d.hi = std::max(w[i].lo, w[i].hi);
    u64 q, r;
    divmod_M(e, d.lo, q, r);
    d.Q = q;
    d.lomod = (u32)r;
    const u64 len = d.hi - d.lo;
    u64 maxpos = 0, rem_;                                // most positions any lane can hold
    if (len) { divmod_M(e, len - 1, maxpos, rem_); ++maxpos; }
    d.item0 = items;
    d.G = 1; d.lane0 = 0;
    if (maxpos <= e->sched.short_max) {
      d.seg = SEG_SMALL; d.nseg = 0; d.groups = 0;
      if (maxpos) {
        // Shorter than M: only the classes in [lo mod M, lo mod M + len) have a position,
        // a contiguous lane range unless it wraps past M.
        u64 la = 0, lb = L;
        if (len < M && d.lomod + len <= M) {
          la = classes_below(e, d.lomod);
          lb = classes_below(e, d.lomod + len);
        }
        if (la < lb) {
          u64 lq, lr;
          divmod_M(e, len, lq, lr);
          shortw.push_back(ShortWin{d.Q, d.lomod, (u32)i, (u32)la, (u32)lb, (u32)lq, (u32)lr});
        }
      }
    } else {
      d.seg = SEG_BIG; d.nseg = (u32)((maxpos + SEG_BIG - 1) / SEG_BIG); d.groups = (u32)L;
    }
    items += (u64)d.groups * d.nseg;
  }
  return items;
}

// Wheel positions in [lo, hi): L per full period of M, plus the classes among the residues
// of the remainder (the sum over lanes of sieve/rung_scan3.cpp:716's npos).
static u64 positions_in(const es_engine *e, u64 lo, u64 hi) {
  if (hi <= lo) return 0;
  const u64 M = e->M;
  u64 qa, a, ql, rem;
  divmod_M(e, lo, qa, a);
  divmod_M(e, hi - lo, ql, rem);
  u64 part = a + rem <= M ? classes_below(e, a + rem) - classes_below(e, a)
                          : (e->classes.size() - classes_below(e, a)) + classes_below(e, a + rem - M);
  return ql * e->classes.size() + part;
}

// One pass of the funnel on the engine's stream: reset the counters, copy the batch header
// and descriptors from pinned staging (ncopy windows), the marking kernels, the survivor
// tail, and the copies of the run counters back to pinned memory. With `capture` the event
// records are external graph nodes, so that the kernels can still be timed when the
// sequence runs as a graph. `items_hint` sizes k_mark's grid for the plain schedule.
// The funnel's front on the slot's stream: run counters cleared, batch header and window
// descriptors copied in, residues, marking (short and long windows), Miller-Rabin.
static es_status enqueue_front(es_engine *e, Slot *sl, bool persistent, WinCount *cnt, size_t ncopy, size_t nshort_copy,
                               u64 items_hint, bool capture) {
  MarkParams P = mark_params(e, sl);
  TailParams T = tail_params(e, sl);
  P.cnt = cnt;
  T.cnt = cnt;
  cudaStream_t st = sl->stream;
  auto rec = [&](int k) {
    return capture ? cudaEventRecordWithFlags(sl->ev[k], st, cudaEventRecordExternal) : cudaEventRecord(sl->ev[k], st);
  };
  CU(cudaMemsetAsync(sl->d_ctr, 0, CTR_BYTES, st));
  CU(cudaMemsetAsync(sl->d_status, 0, sizeof(u32), st));
  CU(cudaMemcpyAsync(sl->d_hdr, sl->h_hdr, sizeof(BatchHdr), cudaMemcpyHostToDevice, st));
  CU(cudaMemcpyAsync(sl->d_win, sl->h_win, ncopy * sizeof(WinDev), cudaMemcpyHostToDevice, st));
  if (nshort_copy) CU(cudaMemcpyAsync(sl->d_shortw, sl->h_short, nshort_copy * sizeof(ShortWin), cudaMemcpyHostToDevice, st));
  CU(rec(0));
  k_prep<<<e->sm_count * 4, 256, 0, st>>>(sl->d_hdr, sl->d_win, e->d_sdist, e->D, e->Dq, sl->d_Qm);
  CU(cudaGetLastError());
  CU(rec(7));
  {
    ShortParams S;
    S.rho = e->d_rho; S.K0 = e->d_K0; S.fdesc = e->d_fdesc; S.Qm = sl->d_Qm; S.mtab = e->d_mtab;
    S.mdesc = e->d_mdesc; S.lfil = e->d_lfil; S.win = sl->d_win; S.shortw = sl->d_shortw;
    S.surv = sl->d_surv; S.surv_count = sl->d_ctr + 1; S.cnt = cnt; S.surv_cap = sl->cap; S.M = e->M;
    S.L = (u32)e->classes.size(); S.ldk = e->ldk; S.D = e->D; S.Dq = e->Dq; S.Wpad = e->Wpad; S.hdr = sl->d_hdr;
    S.nm_cov = e->nm_cov; S.nm_all = e->nm_all; S.nl_cov = e->nl_cov; S.nl_all = e->nl_all;
    k_mark_short<SHORT_BLOCK><<<(S.L + SHORT_LANES - 1) / SHORT_LANES, SHORT_BLOCK, short_smem(e), st>>>(S);
    CU(cudaGetLastError());
  }
  CU(rec(8));
  const unsigned grid = persistent ? (unsigned)((u64)e->sm_count * e->mark_occupancy)
                                   : (unsigned)std::max<u64>(1, std::min<u64>(items_hint, 0x7FFFFFFFull));
  k_mark<MARK_BLOCK><<<grid, MARK_BLOCK, mark_smem(e), st>>>(P, persistent ? 1 : 0);
  CU(cudaGetLastError());
  CU(rec(1));
  k_mr<<<e->sm_count * ES_MR_BLOCKS_PER_SM, 256, 0, st>>>(T);
  CU(cudaGetLastError());
  k_mr2<<<e->sm_count * 2, 256, 0, st>>>(T);
  CU(cudaGetLastError());
  CU(rec(2));
  return ES_OK;
}

// The funnel's tail on the slot's stream: stage D, stage E, run counters and status copied out.
static es_status enqueue_tail(es_engine *e, Slot *sl, WinCount *cnt, bool capture) {
  TailParams T = tail_params(e, sl);
  T.cnt = cnt;
  cudaStream_t st = sl->stream;
  auto rec = [&](int k) {
    return capture ? cudaEventRecordWithFlags(sl->ev[k], st, cudaEventRecordExternal) : cudaEventRecord(sl->ev[k], st);
  };
  k_rung<<<e->sm_count * e->sched.rung_blocks_per_sm, RUNG_WARPS * 32, 0, st>>>(T, (e->flags & ES_FLAG_NO_RUNG) ? 1 : 0);
  CU(cudaGetLastError());
  CU(rec(3));
  k_direct<<<e->sm_count, 32, 0, st>>>(T);
  CU(cudaGetLastError());
  CU(rec(4));
  CU(cudaMemcpyAsync(sl->h_ctr, sl->d_ctr, 8 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
  CU(cudaMemcpyAsync(sl->h_status, sl->d_status, sizeof(u32), cudaMemcpyDeviceToHost, st));
  return ES_OK;
}

// The persistent schedule as a CUDA graph: counters cleared, the whole staging area copied,
// every kernel, and the counters copied back, captured once and replayed per batch.
constexpr size_t REC_PREFIX = 4096;

static es_status capture_graph(es_engine *e, Slot *sl) {
  drop_graph(sl);
  // the front: per-window counters cleared, then the funnel up to Miller-Rabin
  CU(cudaStreamBeginCapture(sl->stream, cudaStreamCaptureModeThreadLocal));
  es_status s = ES_OK;
  const cudaError_t m = cudaMemsetAsync(sl->d_cnt, 0, sl->win_cap * sizeof(WinCount), sl->stream);
  if (m == cudaSuccess) s = enqueue_front(e, sl, true, sl->d_cnt, sl->win_cap, sl->shortw_cap, 0, true);
  cudaGraph_t g = nullptr;
  cudaError_t end = cudaStreamEndCapture(sl->stream, &g);
  if (m != cudaSuccess) return fail(e, ES_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(m));
  if (s != ES_OK) { if (g) cudaGraphDestroy(g); return s; }
  if (end != cudaSuccess) return fail(e, ES_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(end));
  sl->graph = g;
  CU(cudaGraphInstantiate(&sl->gexec, g, 0));
  // the tail: stage D and E, then the counters and the first REC_PREFIX record slots copied
  // back, so that a batch with fewer records (every 4096-window batch at 1e19 has about
  // 1.6 K) needs no copy after the run
  CU(cudaStreamBeginCapture(sl->stream, cudaStreamCaptureModeThreadLocal));
  s = enqueue_tail(e, sl, sl->d_cnt, true);
  sl->rec_prefix = std::min<size_t>(sl->cap, REC_PREFIX);
  if (s == ES_OK) {
    cudaError_t c2 = cudaMemcpyAsync(sl->h_cnt, sl->d_cnt, sl->win_cap * sizeof(WinCount),
                                     cudaMemcpyDeviceToHost, sl->stream);
    if (c2 == cudaSuccess)
      c2 = cudaMemcpyAsync(sl->h_recs, sl->d_recs, sl->rec_prefix * sizeof(RecDev), cudaMemcpyDeviceToHost, sl->stream);
    if (c2 != cudaSuccess) s = fail(e, ES_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(c2));
  }
  g = nullptr;
  end = cudaStreamEndCapture(sl->stream, &g);
  if (s != ES_OK) { if (g) cudaGraphDestroy(g); return s; }
  if (end != cudaSuccess) return fail(e, ES_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(end));
  sl->graph2 = g;
  CU(cudaGraphInstantiate(&sl->gexec2, g, 0));
  return ES_OK;
}

// Launches a captured persistent run on the slot's stream. The front waits for the front
// most recently launched on any other slot, so batches are marked one at a time in launch
// order, and a batch's stage-D tail (a few latency-bound factorizations on a handful of SMs)
// runs beside the next batch's marking instead of leaving the GPU idle.
static es_status launch_persistent(es_engine *e, Slot *sl) {
  {
    std::lock_guard<std::mutex> lk(e->front_mu);
    if (e->last_front && e->last_front != sl) CU(cudaStreamWaitEvent(sl->stream, e->last_front->ev[11], 0));
    CU(cudaGraphLaunch(sl->gexec, sl->stream));
    CU(cudaEventRecord(sl->ev[11], sl->stream));
    e->last_front = sl;
  }
  CU(cudaGraphLaunch(sl->gexec2, sl->stream));
  return ES_OK;
}

static float ev_ms(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0;
  if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess) { (void)cudaGetLastError(); ms = 0; }
  return ms;
}

static std::string status_text(u32 st) {
  std::string s;
  if (st & ST_RHO_BUDGET) s += " rho-budget";
  if (st & ST_FAC_OVERFLOW) s += " factor-overflow";
  if (st & ST_STACK_OVERFLOW) s += " factor-stack";
  if (st & ST_QUEUE_TIMEOUT) s += " queue-timeout";
  if (st & ST_BAD_INPUT) s += " bad-input";
  if (st & ST_CERT_BAD) s += " certificate-self-check";
  return s;
}

// Runs windows through the funnel and collects counters and sorted records. Re-runs
// with larger buffers when the survivor list overflowed (the count is exact even then).
static double ms_since(std::chrono::steady_clock::time_point t) {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t).count();
}

static es_status run_device_windows(es_engine *e, Slot *sl, const es_window *w, size_t n, int schedule,
                                    es_counters *per_window, es_records *recs) {
  const auto t_start = std::chrono::steady_clock::now();
  double setup_ms = 0, device_ms = 0;
  const u64 floor_ = std::max(e->wheel_pmin, e->cover_pmax);
  for (size_t i = 0; i < n; ++i) {
    if (w[i].hi > DIRECT_PMAX)
      return fail(e, ES_ERR_RANGE, "HI must not exceed the stage-E ceiling " + std::to_string(DIRECT_PMAX));
    if (w[i].lo <= floor_)
      return fail(e, ES_ERR_RANGE, "LO must exceed max pmin of the filter table (" + std::to_string(floor_) + ")");
  }
  std::vector<WinDev> &wd = sl->hs.wd;
  std::vector<ShortWin> &shortw = sl->hs.shortw;
  const u64 total_items = describe(e, w, n, wd, shortw);
  std::vector<u64> &npos = sl->hs.npos;
  npos.resize(n);
  u64 positions_bound = 0;
  for (size_t i = 0; i < n; ++i) positions_bound += (npos[i] = positions_in(e, w[i].lo, w[i].hi));
  size_t cap = (size_t)std::min<u64>(std::max<u64>(positions_bound / 64, 1 << 16), 1ull << 26);
  cap = std::max(cap, sl->cap);
  const bool persistent = schedule == ES_SCHED_PERSISTENT;
  std::vector<RecDev> &hr = sl->hs.hr;
  hr.clear();
  bool done = false;
  for (int attempt = 0; attempt < 4 && !done; ++attempt) {
    es_status s = ensure_capacity(e, sl, n, cap);
    if (s) return s;
    double mark_ms = 0, mr_ms = 0, rung_ms = 0, direct_ms = 0, prep_ms = 0, short_ms = 0, long_ms = 0;
    u64 launches = 0, surv_max = 0, surv_total = 0, prime_total = 0;
    u32 status = 0;
    hr.clear();
    size_t have_recs = 0;                 // records already on the host (the graph's prefix copy)
    auto collect = [&]() -> es_status {   // after a pass: timings, counts, records
      prep_ms += ev_ms(sl->ev[0], sl->ev[7]); short_ms += ev_ms(sl->ev[7], sl->ev[8]);
      long_ms += ev_ms(sl->ev[8], sl->ev[1]);
      mark_ms += ev_ms(sl->ev[0], sl->ev[1]); mr_ms += ev_ms(sl->ev[1], sl->ev[2]);
      rung_ms += ev_ms(sl->ev[2], sl->ev[3]); direct_ms += ev_ms(sl->ev[3], sl->ev[4]);
      const unsigned long long *ctr = sl->h_ctr;
      surv_max = std::max<u64>(surv_max, ctr[1]);
      surv_total += ctr[1]; prime_total += ctr[2];
      status |= *sl->h_status;
      if (ctr[1] > sl->cap) return ES_OK;
      const size_t nrec = (size_t)std::min<u64>(ctr[4], sl->cap);
      const size_t have = std::min(nrec, have_recs);
      if (nrec > have) {
        CU(cudaMemcpyAsync(sl->h_recs + have, sl->d_recs + have, (nrec - have) * sizeof(RecDev),
                           cudaMemcpyDeviceToHost, sl->stream));
        CU(cudaStreamSynchronize(sl->stream));
      }
      if (nrec) hr.insert(hr.end(), sl->h_recs, sl->h_recs + nrec);
      return ES_OK;
    };
    if (persistent) {
      sl->h_hdr->total_items = total_items;
      sl->h_hdr->nwin = (u32)n;
      sl->h_hdr->nshort = (u32)shortw.size();
      memcpy(sl->h_win, wd.data(), n * sizeof(WinDev));
      if (!shortw.empty()) {
        // largest first: the warps of a k_mark_short CTA deal the windows round robin, so the
        // CTA's last window is a small one
        // a counting sort on the work's binary order of magnitude (largest first, ties in
        // input order) is all the balance needs
        const size_t ns = shortw.size();
        std::vector<uint8_t> &mag = sl->hs.mag;
        mag.resize(ns);
        u32 start[34] = {0};
        for (size_t k = 0; k < ns; ++k) {
          const ShortWin &x = shortw[k];
          const u64 work = (u64)(x.lb - x.la) * (x.lq + 1);          // < 2^21
          mag[k] = (uint8_t)(32 - __builtin_clz((u32)work | 1u));    // 1 .. 22
          ++start[33 - mag[k]];
        }
        for (int b = 1; b < 34; ++b) start[b] += start[b - 1];
        for (size_t k = 0; k < ns; ++k) sl->h_short[start[32 - mag[k]]++] = shortw[k];
      }
      if (!sl->gexec || !sl->gexec2) { s = capture_graph(e, sl); if (s) return s; }
      setup_ms = ms_since(t_start);
      const auto t_launch = std::chrono::steady_clock::now();
      s = launch_persistent(e, sl);
      if (s) return s;
      CU(cudaStreamSynchronize(sl->stream));
      device_ms = ms_since(t_launch);
      launches = 7;
      have_recs = sl->rec_prefix;
      s = collect();
      if (s) return s;
    } else {
      // The plain schedule: the same kernels, one launch sequence per window.
      CU(cudaMemsetAsync(sl->d_cnt, 0, n * sizeof(WinCount), sl->stream));
      size_t k = 0;                      // next short-window entry (describe emits them in order)
      for (size_t i = 0; i < n; ++i) {
        sl->h_win[0] = wd[i];
        sl->h_win[0].item0 = 0;
        const u64 items = (u64)wd[i].nseg * wd[i].groups;
        u32 nshort = 0;
        if (k < shortw.size() && shortw[k].wi == i) { sl->h_short[0] = shortw[k++]; sl->h_short[0].wi = 0; nshort = 1; }
        sl->h_hdr->total_items = items; sl->h_hdr->nwin = 1; sl->h_hdr->nshort = nshort;
        s = enqueue_front(e, sl, false, sl->d_cnt + i, 1, nshort, items, false);
        if (s) return s;
        s = enqueue_tail(e, sl, sl->d_cnt + i, false);
        if (s) return s;
        CU(cudaStreamSynchronize(sl->stream));
        launches += 7;
        const size_t base = hr.size();
        s = collect();
        if (s) return s;
        if (surv_max > sl->cap) break;
        for (size_t r = base; r < hr.size(); ++r) hr[r].win = (u32)i;
      }
      CU(cudaMemcpyAsync(sl->h_cnt, sl->d_cnt, n * sizeof(WinCount), cudaMemcpyDeviceToHost, sl->stream));
      CU(cudaStreamSynchronize(sl->stream));
    }
    if (surv_max > sl->cap) {            // overflow: grow to the exact need and re-run
      cap = (size_t)(surv_max + surv_max / 4 + 1024);
      continue;
    }
    if (status) return fail(e, ES_ERR_DEVICE_STATUS, "device status:" + status_text(status));
    sl->timing.total_ms = mark_ms + mr_ms + rung_ms + direct_ms;   // kernels only, inputs resident
    sl->timing.mark_ms = mark_ms; sl->timing.mr_ms = mr_ms;
    sl->timing.prep_ms = prep_ms; sl->timing.mark_short_ms = short_ms; sl->timing.mark_long_ms = long_ms;
    sl->timing.short_pairs = (u64)shortw.size() * e->classes.size();
    sl->timing.mask_bytes = shortw.empty() ? 0 : (u64)e->classes.size() * e->Wpad * 8;
    sl->timing.rung_ms = rung_ms; sl->timing.direct_ms = direct_ms;
    sl->timing.marks_kernel_launches = persistent ? 1 : n;
    sl->timing.kernel_launches = launches;
    sl->timing.mark_items = total_items;
    sl->timing.survivors = surv_total;
    sl->timing.primes = prime_total;
    done = true;
  }
  if (!done) return fail(e, ES_ERR_NOMEM, "survivor list kept overflowing");
  for (size_t i = 0; i < n; ++i) {      // the SUMMARY counters (sieve/rung_scan3.cpp:764-772)
    const WinCount &c = sl->h_cnt[i];
    es_counters &o = per_window[i];
    o.positions = npos[i];
    if (e->nf == e->ncov) { o.covered = o.positions - c.surv; o.sieved = 0; }
    else { o.covered = o.positions - c.after_covers; o.sieved = c.after_covers - c.surv; }
    // every prime survivor ends as a rung record, a direct one or an unsolved one, so the
    // composites are the rest (a run where that fails is refused by its status)
    const unsigned long long primes_w = c.rung + c.direct + c.unsolved;
    o.mr = c.surv; o.composite = c.surv >= primes_w ? c.surv - primes_w : 0; o.rung = c.rung; o.direct = c.direct;
    o.survivors = c.unsolved;
  }
  if (recs) {
    // Lane-major order within each window: a counting sort on the window index straight into
    // the caller's buffer, then (lane, J) order inside each window's few records.
    static_assert(sizeof(RecDev) == sizeof(es_record), "record layout");
    recs->n = hr.size();
    recs->recs = (es_record *)malloc(std::max<size_t>(hr.size(), 1) * sizeof(es_record));
    if (!recs->recs) return fail(e, ES_ERR_NOMEM, "host records");
    RecDev *out = reinterpret_cast<RecDev *>(recs->recs);
    std::vector<u32> &start = sl->hs.start, &pos = sl->hs.pos;
    start.assign(n + 1, 0);
    for (const RecDev &r : hr) ++start[std::min<size_t>(r.win, n - 1) + 1];
    for (size_t i = 0; i < n; ++i) start[i + 1] += start[i];
    pos.assign(start.begin(), start.end() - 1);
    for (const RecDev &r : hr) out[pos[std::min<size_t>(r.win, n - 1)]++] = r;
    for (size_t i = 0; i < n; ++i) {
      if (start[i + 1] - start[i] > 1)
        std::sort(out + start[i], out + start[i + 1], [](const RecDev &a, const RecDev &b) {
          if (a.win != b.win) return a.win < b.win;
          if (a.lane != b.lane) return a.lane < b.lane;
          return a.J < b.J;
        });
    }
  }
  sl->timing.host_setup_ms = setup_ms;
  sl->timing.host_device_ms = device_ms;
  sl->timing.host_collect_ms = ms_since(t_start) - setup_ms - device_ms;
  return ES_OK;
}

// Windows whose lanes hold more than short_max positions are, by default, cut into
// sub-windows of short_max positions per lane (short_max * M integers; the last one
// shorter), which the short-window kernel marks with its early exit; with long_split = 0
// they keep one device window each and go to the segment marking. Sub-window t of a window
// starts t * short_max positions into every lane, so its records map back to the window by
// J += t * short_max, and its counters add up to the window's (every counter is a sum over
// positions). Device windows are run in passes of at most PASS_WINDOWS. Every caller passes
// per_window zeroed.
constexpr size_t PASS_WINDOWS = 1u << 18;

static es_status run_windows(es_engine *e, Slot *sl, const es_window *w, size_t n, int schedule,
                             es_counters *per_window, es_records *recs) {
  const u64 M = e->M, S = e->sched.short_max;
  const u64 floor_ = std::max(e->wheel_pmin, e->cover_pmax);
  bool split = false;
  for (size_t i = 0; i < n; ++i) {                 // refuse what a run would refuse, first
    if (w[i].hi > DIRECT_PMAX)
      return fail(e, ES_ERR_RANGE, "HI must not exceed the stage-E ceiling " + std::to_string(DIRECT_PMAX));
    if (w[i].lo <= floor_)
      return fail(e, ES_ERR_RANGE, "LO must exceed max pmin of the filter table (" + std::to_string(floor_) + ")");
    const u64 len = w[i].hi > w[i].lo ? w[i].hi - w[i].lo : 0;
    // more than S positions per lane; the plain schedule keeps one launch sequence per window
    if (e->sched.long_split && schedule == ES_SCHED_PERSISTENT && len > S * M) split = true;
  }
  if (!split) return run_device_windows(e, sl, w, n, schedule, per_window, recs);
  std::vector<es_record> &all = sl->hs.all;
  all.clear();
  es_timing_t tot{};
  std::vector<es_window> &dw = sl->hs.dw;
  std::vector<std::pair<u32, u64>> &dmap = sl->hs.dmap;   // (window, position offset) per device window
  std::vector<es_counters> &pc = sl->hs.pc;
  dw.reserve(PASS_WINDOWS);
  dmap.reserve(PASS_WINDOWS);
  // device windows are produced a pass at a time: (i, t) is the next sub-window to emit
  size_t i = 0;
  u64 t = 0;
  while (i < n) {
    dw.clear();
    dmap.clear();
    while (i < n && dw.size() < PASS_WINDOWS) {
      const u64 lo = w[i].lo, hi = std::max(w[i].lo, w[i].hi);
      const u64 len = hi - lo;
      if (!e->sched.long_split || len <= S * M) {
        dw.push_back({lo, hi});
        dmap.push_back({(u32)i, 0});
        ++i;
        continue;
      }
      const u64 step = S * M, a = lo + t * step;  // t * step < len: no overflow
      dw.push_back({a, a + std::min(step, hi - a)});
      dmap.push_back({(u32)i, t * S});
      if (hi - a <= step) { ++i; t = 0; } else ++t;
    }
    const size_t m = dw.size();
    pc.resize(m);
    es_records pr{nullptr, 0};
    const es_status st = run_device_windows(e, sl, dw.data(), m, schedule, pc.data(), recs ? &pr : nullptr);
    if (st != ES_OK) { es_free_records(&pr); return st; }
    for (size_t k = 0; k < m; ++k) {
      es_counters &o = per_window[dmap[k].first];
      const es_counters &c = pc[k];
      o.positions += c.positions; o.covered += c.covered; o.sieved += c.sieved; o.mr += c.mr;
      o.composite += c.composite; o.rung += c.rung; o.direct += c.direct; o.survivors += c.survivors;
    }
    all.reserve(all.size() + pr.n);
    for (size_t r = 0; r < pr.n; ++r) {
      es_record x = pr.recs[r];
      const auto &mp = dmap[x.window];
      x.window = mp.first;
      x.J += mp.second;
      all.push_back(x);
    }
    es_free_records(&pr);
    const es_timing_t &tt = sl->timing;
    tot.total_ms += tt.total_ms; tot.mark_ms += tt.mark_ms; tot.mr_ms += tt.mr_ms; tot.rung_ms += tt.rung_ms;
    tot.direct_ms += tt.direct_ms; tot.prep_ms += tt.prep_ms; tot.mark_short_ms += tt.mark_short_ms;
    tot.mark_long_ms += tt.mark_long_ms; tot.marks_kernel_launches += tt.marks_kernel_launches;
    tot.kernel_launches += tt.kernel_launches; tot.mark_items += tt.mark_items; tot.survivors += tt.survivors;
    tot.primes += tt.primes; tot.short_pairs += tt.short_pairs; tot.mask_bytes += tt.mask_bytes;
    tot.host_setup_ms += tt.host_setup_ms; tot.host_device_ms += tt.host_device_ms;
    tot.host_collect_ms += tt.host_collect_ms;
  }
  sl->timing = tot;
  if (recs) {
    // Each pass's records come in (device window, lane, J) order and the device windows of a
    // window are consecutive (across passes too), so the records are already grouped by window
    // in ascending order; only a split window's group needs putting back in (lane, J) order.
    for (size_t a = 0; a < all.size();) {
      size_t b = a + 1;
      while (b < all.size() && all[b].window == all[a].window) ++b;
      if (b - a > 1)
        std::sort(all.begin() + a, all.begin() + b, [](const es_record &x, const es_record &y) {
          if (x.lane != y.lane) return x.lane < y.lane;
          return x.J < y.J;
        });
      a = b;
    }
    recs->n = all.size();
    recs->recs = (es_record *)malloc(std::max<size_t>(all.size(), 1) * sizeof(es_record));
    if (!recs->recs) return fail(e, ES_ERR_NOMEM, "host records");
    memcpy(recs->recs, all.data(), all.size() * sizeof(es_record));
  }
  return ES_OK;
}

static es_status build_tables(es_engine *e) {
  const u64 M = e->M;
  const u32 L = (u32)e->classes.size();
  const size_t nf = e->mods.size();
  // Per filter: g = gcd(M, mod), s = mod/g, inv = ((M/g) mod s)^-1 mod s.
  std::vector<u32> g(nf), s(nf), inv(nf);
  for (size_t i = 0; i < nf; ++i) {
    const u64 mod = e->mods[i];
    if (mod == 0) return fail(e, ES_ERR_FILTERS, "filter with modulus 0");
    if (mod > 0xFFFFFFFFull) return fail(e, ES_ERR_ARG, "filter modulus above 2^32 is not supported");
    const u64 gg = gcd_u64(M, mod), ss = mod / gg;
    if (ss > 0xFFFFull) return fail(e, ES_ERR_ARG, "filter stride mod/gcd(M,mod) above 65535 is not supported");
    bool ok;
    const u64 iv = ss == 1 ? 0 : inv_mod((M / gg) % ss, ss, ok);
    if (ss != 1 && !ok) return fail(e, ES_ERR_ARG, "non-invertible stride (impossible for g = gcd)");
    g[i] = (u32)gg; s[i] = (u32)ss; inv[i] = (u32)iv;
  }
  // Marking order: by stride within each phase, so that a warp's 32 filters have similar
  // trip counts. Marking is idempotent, so the order cannot change the result.
  e->order.resize(nf);
  for (size_t i = 0; i < nf; ++i) e->order[i] = (u32)i;
  std::stable_sort(e->order.begin(), e->order.begin() + e->ncov, [&](u32 a, u32 b) { return s[a] < s[b]; });
  std::stable_sort(e->order.begin() + e->ncov, e->order.end(), [&](u32 a, u32 b) { return s[a] < s[b]; });
  std::vector<u32> sd;
  for (size_t i = 0; i < nf; ++i) sd.push_back(s[i]);
  std::sort(sd.begin(), sd.end());
  sd.erase(std::unique(sd.begin(), sd.end()), sd.end());
  if (sd.size() > (size_t)DMAX) return fail(e, ES_ERR_ARG, "more than 8192 distinct filter strides");
  e->D = (u32)sd.size();
  e->Dq = (e->D + 7) & ~7u;                        // Qm rows: whole 16-byte chunks
  std::vector<u64> om(nf), orr(nf);
  std::vector<u32> og(nf), oinv(nf), fdesc(nf);
  for (size_t k = 0; k < nf; ++k) {
    const u32 i = e->order[k];
    om[k] = e->mods[i]; orr[k] = e->ress[i]; og[k] = g[i]; oinv[k] = inv[i];
    const u32 di = (u32)(std::lower_bound(sd.begin(), sd.end(), s[i]) - sd.begin());
    fdesc[k] = s[i] | (di << 16);
  }
  e->nf = (u32)nf;
  e->ldk = (u32)((nf + 7) & ~7ull);
  std::vector<u32> rho(L);
  for (u32 l = 0; l < L; ++l) rho[l] = (u32)e->classes[l];
  // trial-division table
  std::vector<u32> tdp;
  std::vector<TdEntry> tde;
  {
    std::vector<uint8_t> comp(65537, 0);
    for (u64 i = 2; i <= 65536; ++i) {
      if (comp[i]) continue;
      for (u64 j = i * i; j <= 65536; j += i) comp[j] = 1;
      if (i == 2) continue;
      u64 x = i;
      for (int k = 0; k < 5; ++k) x *= 2 - i * x;
      tdp.push_back((u32)i);
      tde.push_back(TdEntry{x, ~0ull / i});
    }
    if ((int)tdp.size() != NTD) return fail(e, ES_ERR_ARG, "trial-division table size");
  }
  // temporaries of the table build, freed on every return path
  struct Temps {
    void *p[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    ~Temps() { for (void *x : p) cudaFree(x); }
  } temps;
  u64 *d_mods = nullptr, *d_ress = nullptr;
  u32 *d_g = nullptr, *d_inv = nullptr;
  CU(cudaMalloc(&e->d_rho, L * sizeof(u32)));
  CU(cudaMalloc(&e->d_fdesc, std::max<size_t>(nf, 1) * sizeof(u32)));
  CU(cudaMalloc(&e->d_sdist, std::max<size_t>(sd.size(), 1) * sizeof(u32)));
  CU(cudaMalloc(&e->d_K0, (size_t)L * e->ldk * sizeof(u16)));
  CU(cudaMalloc(&e->d_tdp, tdp.size() * sizeof(u32)));
  CU(cudaMalloc(&e->d_tde, tde.size() * sizeof(TdEntry)));
  CU(cudaMalloc(&e->d_tdi, tde.size() * sizeof(u64)));
  CU(cudaMalloc(&e->d_tdqm, tdp.size() * sizeof(uint2)));
  CU(cudaMalloc(&d_mods, std::max<size_t>(nf, 1) * sizeof(u64)));
  temps.p[0] = d_mods;
  CU(cudaMalloc(&d_ress, std::max<size_t>(nf, 1) * sizeof(u64)));
  temps.p[1] = d_ress;
  CU(cudaMalloc(&d_g, std::max<size_t>(nf, 1) * sizeof(u32)));
  temps.p[2] = d_g;
  CU(cudaMalloc(&d_inv, std::max<size_t>(nf, 1) * sizeof(u32)));
  temps.p[3] = d_inv;
  // The table copies go on the stream the build kernels run on (slot 0's, non-blocking, so not
  // ordered after the legacy stream); the host vectors they read outlive the synchronisation
  // at the end of this function.
  cudaStream_t bs = e->slots[0].stream;
  CU(cudaMemcpyAsync(e->d_rho, rho.data(), L * sizeof(u32), cudaMemcpyHostToDevice, bs));
  CU(cudaMemcpyAsync(e->d_fdesc, fdesc.data(), nf * sizeof(u32), cudaMemcpyHostToDevice, bs));
  CU(cudaMemcpyAsync(e->d_sdist, sd.data(), sd.size() * sizeof(u32), cudaMemcpyHostToDevice, bs));
  CU(cudaMemcpyAsync(e->d_tdp, tdp.data(), tdp.size() * sizeof(u32), cudaMemcpyHostToDevice, bs));
  CU(cudaMemcpyAsync(e->d_tde, tde.data(), tde.size() * sizeof(TdEntry), cudaMemcpyHostToDevice, bs));
  std::vector<u64> tdi(tde.size());
  for (size_t i = 0; i < tde.size(); ++i) tdi[i] = tde[i].inv;
  CU(cudaMemcpyAsync(e->d_tdi, tdi.data(), tdi.size() * sizeof(u64), cudaMemcpyHostToDevice, bs));
  std::vector<uint2> tdqm(tdp.size());
  for (size_t i = 0; i < tdp.size(); ++i) tdqm[i] = make_uint2(tdp[i], (u32)((1ull << 32) / tdp[i]));
  CU(cudaMemcpyAsync(e->d_tdqm, tdqm.data(), tdqm.size() * sizeof(uint2), cudaMemcpyHostToDevice, bs));
  CU(cudaMemcpyAsync(d_mods, om.data(), nf * sizeof(u64), cudaMemcpyHostToDevice, bs));
  CU(cudaMemcpyAsync(d_ress, orr.data(), nf * sizeof(u64), cudaMemcpyHostToDevice, bs));
  CU(cudaMemcpyAsync(d_g, og.data(), nf * sizeof(u32), cudaMemcpyHostToDevice, bs));
  CU(cudaMemcpyAsync(d_inv, oinv.data(), nf * sizeof(u32), cudaMemcpyHostToDevice, bs));
  const u64 total = (u64)L * e->ldk;
  k_build_k0<<<(unsigned)((total + 255) / 256), 256, 0, bs>>>(e->d_rho, L, d_mods, d_ress, d_g, d_inv,
                                                              e->d_fdesc, (u32)nf, e->ldk, e->d_K0);
  CU(cudaGetLastError());
  // Kill masks for short windows: within each phase (covers, then stage-B' primes), the
  // smallest strides get a mask while the per-lane table fits MASK_BYTES_MAX; the filters of
  // the remaining strides are checked one by one from the first-hit table. The masked strides
  // are then ordered by how many positions they kill -- the sum over lanes and filters of
  // 1/s where the filter hits the lane (rho == res mod g) -- so that k_mark_short, which stops
  // once a segment is dead, meets the densest strides first. Kills are ORed, so the order
  // cannot change a result.
  {
    std::vector<MaskDesc> md;
    std::vector<int> fmask(nf, -1);
    std::vector<u32> lfil_cov, lfil_siv;
    std::map<u32, std::unordered_map<u32, u32>> lanes_mod;     // g -> (rho mod g -> lanes)
    for (size_t k = 0; k < nf; ++k) {
      auto &h = lanes_mod[og[k]];
      if (h.empty())
        for (u32 l = 0; l < L; ++l) ++h[rho[l] % og[k]];
    }
    std::vector<double> kills(65536, 0.0);
    for (size_t k = 0; k < nf; ++k) {
      const auto &h = lanes_mod[og[k]];
      const auto it = h.find((u32)(orr[k] % og[k]));
      if (it != h.end()) kills[fdesc[k] & 0xFFFFu] += (double)it->second / (double)(fdesc[k] & 0xFFFFu);
    }
    u32 words = 0;
    for (int phase = 0; phase < 2; ++phase) {
      const size_t f0 = phase ? e->ncov : 0, f1 = phase ? nf : e->ncov;
      std::vector<u32> strides;
      for (size_t k = f0; k < f1; ++k) strides.push_back(fdesc[k] & 0xFFFFu);
      std::sort(strides.begin(), strides.end());
      strides.erase(std::unique(strides.begin(), strides.end()), strides.end());
      std::vector<int> slot_of(65536, -1);
      const size_t m_first = md.size();
      for (u32 st : strides) {
        // bits [0, s + SEG_SMALL) plus one spare word: a segment of up to SEG_SMALL positions
        // starting at any residue below s reads words r/32 .. r/32 + SEG_SMALL/32 of the slice
        const u32 wd = (st + SEG_SMALL + 31) / 32 + 1;
        if ((size_t)(words + wd) * 4 > MASK_BYTES_MAX || md.size() >= SMD_MAX) break;
        const u32 di = (u32)(std::lower_bound(sd.begin(), sd.end(), st) - sd.begin());
        md.push_back(MaskDesc{st, di, words, 0});
        words += wd;
      }
      std::stable_sort(md.begin() + m_first, md.end(),
                       [&](const MaskDesc &x, const MaskDesc &y) { return kills[x.s] > kills[y.s]; });
      for (size_t m = m_first; m < md.size(); ++m) slot_of[md[m].s] = (int)m;
      for (size_t k = f0; k < f1; ++k) {
        const int m = slot_of[fdesc[k] & 0xFFFFu];
        fmask[k] = m;
        if (m < 0) (phase ? lfil_siv : lfil_cov).push_back((u32)k);
      }
      if (phase == 0) e->nm_cov = (u32)md.size();
    }
    e->nm_all = (u32)md.size();
    // Final layout: the first INTERLEAVE_ROUNDS rounds of the covers' phase interleaved (each
    // group of 32 slices padded to its longest), the rest packed; if that no longer fits the
    // per-lane budget, fewer rounds are interleaved (the layout cannot change a result).
    for (u32 rounds = std::min<u32>(INTERLEAVE_ROUNDS, e->nm_cov / 32);; --rounds) {
      const u32 m_inter = 32 * rounds;
      u32 w2 = 0;
      for (u32 g = 0; g < rounds; ++g) {
        u32 maxwd = 0;
        for (u32 j = 0; j < 32; ++j) maxwd = std::max(maxwd, (md[32 * g + j].s + SEG_SMALL + 31) / 32 + 1);
        for (u32 j = 0; j < 32; ++j) { md[32 * g + j].off = w2 + j; md[32 * g + j].sh = 5; }
        w2 += 32 * maxwd;
      }
      for (size_t m = m_inter; m < md.size(); ++m) {
        md[m].off = w2;
        md[m].sh = 0;
        w2 += (md[m].s + SEG_SMALL + 31) / 32 + 1;
      }
      if ((size_t)w2 * 4 <= MASK_BYTES_MAX || rounds == 0) { words = w2; e->m_inter = m_inter; break; }
    }
    e->nl_cov = (u32)lfil_cov.size();
    e->nl_all = (u32)(lfil_cov.size() + lfil_siv.size());
    e->Wpad = std::max<u32>(2, ((words + 1) / 2 + 1) & ~1u);   // in 64-bit words, even
    std::vector<u32> lfil(lfil_cov);
    lfil.insert(lfil.end(), lfil_siv.begin(), lfil_siv.end());
    int *d_fmask = nullptr;
    CU(cudaMalloc(&e->d_mtab, (size_t)L * e->Wpad * sizeof(u64)));
    CU(cudaMalloc(&e->d_mdesc, std::max<size_t>(md.size(), 1) * sizeof(MaskDesc)));
    CU(cudaMalloc(&e->d_lfil, std::max<size_t>(lfil.size(), 1) * sizeof(u32)));
    CU(cudaMalloc(&d_fmask, std::max<size_t>(nf, 1) * sizeof(int)));
    temps.p[4] = d_fmask;
    CU(cudaMemsetAsync(e->d_mtab, 0, (size_t)L * e->Wpad * sizeof(u64), bs));
    if (!md.empty()) CU(cudaMemcpyAsync(e->d_mdesc, md.data(), md.size() * sizeof(MaskDesc), cudaMemcpyHostToDevice, bs));
    if (!lfil.empty()) CU(cudaMemcpyAsync(e->d_lfil, lfil.data(), lfil.size() * sizeof(u32), cudaMemcpyHostToDevice, bs));
    if (nf) CU(cudaMemcpyAsync(d_fmask, fmask.data(), nf * sizeof(int), cudaMemcpyHostToDevice, bs));
    if (nf && !md.empty()) {
      const u64 tt = (u64)L * nf;
      k_build_masks<<<(unsigned)((tt + 255) / 256), 256, 0, e->slots[0].stream>>>(e->d_K0, L, e->ldk, (u32)nf, d_fmask,
                                                                         e->d_mdesc, e->Wpad, e->d_mtab);
      CU(cudaGetLastError());
    }
    CU(cudaStreamSynchronize(bs));
    CU(cudaFuncSetAttribute(k_mark_short<SHORT_BLOCK>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            (int)(SHORT_LANES * (MASK_BYTES_MAX + 16) + SMD_MAX * sizeof(MaskDesc) +
                                  SHORT_HAND_BYTES)));
  }
  CU(cudaStreamSynchronize(e->slots[0].stream));
  // occupancy of the marking kernel, for the persistent grid
  // The attribute is per function and process-wide: set it to the largest size any engine
  // can ask for (DMAX strides), never to this engine's own size, or a second engine with
  // fewer strides would shrink it under the first.
  // Stage D's trial division streams its 78 KB prime table once per factorization: ask for
  // the smallest shared-memory carveout that still holds the resident blocks' static shared
  // memory, so that the rest of the SM's 256 KB stays L1 and the table stays in it.
  {
    int max_smem = 0;
    CU(cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerMultiprocessor, e->device));
    for (const void *f : {(const void *)k_rung, (const void *)k_probe_rung}) {
      cudaFuncAttributes fa;
      CU(cudaFuncGetAttributes(&fa, f));
      const double need = (double)ES_RUNG_MIN_BLOCKS * (fa.sharedSizeBytes + 1024);
      const int pct = std::min(100, (int)(100.0 * need / std::max(max_smem, 1)) + 1);
      CU(cudaFuncSetAttribute(f, cudaFuncAttributePreferredSharedMemoryCarveout, pct));
    }
  }
  const size_t smem = mark_smem(e);
  const size_t smem_max = ((4 * DMAX + 15) & ~15u) + std::max<u32>(SEG_BIG, GROUP * SEG_SMALL) + 16;
  CU(cudaFuncSetAttribute(k_mark<MARK_BLOCK>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_max));
  int occ = 0;
  CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_mark<MARK_BLOCK>, MARK_BLOCK, smem));
  e->mark_occupancy = std::max(occ, 1);
  return ES_OK;
}

constexpr size_t SERVE_QUEUE_WINDOWS = 1 << 20;   // windows waiting, across requests
constexpr size_t SERVE_BATCH_WINDOWS = 8192;      // windows per batch a worker takes

// Device bytes a request's windows need in a slot: descriptors, per-window residues and
// counters, and the survivor-side buffers sized like run_windows sizes them.
static u64 request_bytes(const es_engine *e, const es_window *w, size_t n) {
  u64 pos = 0;
  for (size_t i = 0; i < n; ++i) pos += positions_in(e, w[i].lo, w[i].hi);
  const u64 surv = std::min<u64>(std::max<u64>(pos / 64, 1024), 1ull << 26);
  return n * (sizeof(WinDev) + sizeof(ShortWin) + sizeof(WinCount) + 2ull * e->Dq) +
         surv * (sizeof(Surv) + 3 * sizeof(u32) + sizeof(RecDev));
}

// A serving worker owns slot k: whenever its slot is free it takes every queued request
// that fits one batch (continuous batching -- requests that arrive while other batches run
// join the next one), runs the batch on its own stream, and hands each request its windows'
// counters and records. Workers of different slots run their batches concurrently.
static void serve_worker(es_engine *e, int k) {
  cudaSetDevice(e->device);
  Slot *sl = &e->slots[k];
  for (;;) {
    std::vector<Request *> batch;
    {
      std::unique_lock<std::mutex> lk(e->qmu);
      e->qcv.wait(lk, [&] { return e->stopping || !e->queue.empty(); });
      if (e->stopping && e->queue.empty()) return;
      size_t nw = 0;
      // a solo request (es_submit_batch) is a batch of its own, of any size
      while (!e->queue.empty() &&
             (batch.empty() || (!batch[0]->solo && !e->queue.front()->solo &&
                                nw + e->queue.front()->w.size() <= SERVE_BATCH_WINDOWS))) {
        Request *r = e->queue.front();
        e->queue.pop_front();
        nw += r->w.size();
        e->queued_windows -= r->w.size();
        batch.push_back(r);
      }
    }
    std::vector<es_window> wins;
    for (Request *r : batch) wins.insert(wins.end(), r->w.begin(), r->w.end());
    std::vector<es_counters> cnt(wins.size());
    es_records recs{nullptr, 0};
    es_status st = ES_OK;
    std::string err;
    if (!wins.empty()) {
      std::lock_guard<std::mutex> lk(sl->mu);
      st = run_windows(e, sl, wins.data(), wins.size(), ES_SCHED_PERSISTENT, cnt.data(), &recs);
      if (st != ES_OK) { std::lock_guard<std::mutex> el(e->err_mu); err = e->last_error; }
    }
    // split the batch back into its requests (records are sorted by window)
    size_t w0 = 0, r0 = 0;
    for (Request *r : batch) {
      const size_t n = r->w.size();
      r->st = st;
      r->err = err;
      if (st == ES_OK) {
        r->cnt.assign(cnt.begin() + w0, cnt.begin() + w0 + n);
        size_t r1 = r0;
        while (r1 < recs.n && recs.recs[r1].window < w0 + n) ++r1;
        r->recs.assign(recs.recs + r0, recs.recs + r1);
        for (es_record &x : r->recs) x.window -= (uint32_t)w0;
        r0 = r1;
      }
      w0 += n;
    }
    free(recs.recs);
    {
      std::lock_guard<std::mutex> lk(e->qmu);
      for (Request *r : batch) { r->done = true; e->mem_in_use -= r->mem; }
    }
    e->dcv.notify_all();
  }
}

}  // namespace es

using namespace es;

namespace es {
// Probes: copy in, one kernel, copy out. Small and synchronous.
template <typename Launch>
static es_status probe(es_engine *e, Slot *sl, size_t count, size_t in_bytes, const void *in, size_t out_bytes,
                       std::vector<std::pair<void *, size_t>> outs, Launch launch) {
  std::lock_guard<std::mutex> lk(sl->mu);
  cudaSetDevice(e->device);
  void *d_in = nullptr;
  std::vector<void *> d_outs(outs.size(), nullptr);
  struct Release {                                   // the probe's buffers, on every return path
    void *&in;
    std::vector<void *> &outs;
    ~Release() {
      cudaFree(in);
      for (void *p : outs) cudaFree(p);
    }
  } release{d_in, d_outs};
  (void)out_bytes;
  CU(cudaMalloc(&d_in, std::max<size_t>(in_bytes, 8)));
  for (size_t i = 0; i < outs.size(); ++i) CU(cudaMalloc(&d_outs[i], std::max<size_t>(outs[i].second, 8)));
  // Every copy is queued on the probe's own stream (a non-blocking stream is not ordered after
  // the legacy stream that a plain cudaMemcpy uses), and the host waits for that stream before
  // it reads anything back.
  CU(cudaMemcpyAsync(d_in, in, in_bytes, cudaMemcpyHostToDevice, sl->stream));
  CU(cudaMemsetAsync(sl->d_status, 0, sizeof(u32), sl->stream));
  CU(cudaEventRecord(sl->ev[9], sl->stream));
  launch(d_in, d_outs);
  CU(cudaGetLastError());
  CU(cudaEventRecord(sl->ev[10], sl->stream));
  for (size_t i = 0; i < outs.size(); ++i)
    CU(cudaMemcpyAsync(outs[i].first, d_outs[i], outs[i].second, cudaMemcpyDeviceToHost, sl->stream));
  u32 st = 0;
  CU(cudaMemcpyAsync(&st, sl->d_status, sizeof st, cudaMemcpyDeviceToHost, sl->stream));
  CU(cudaStreamSynchronize(sl->stream));
  sl->timing.total_ms = ev_ms(sl->ev[9], sl->ev[10]);   // the probe kernel alone
  (void)count;
  if (st) return fail(e, ES_ERR_DEVICE_STATUS, "device status:" + status_text(st));
  return ES_OK;
}

}  // namespace es

// ============================================================================ C ABI

extern "C" {

const char *es_status_str(es_status s) {
  switch (s) {
    case ES_OK: return "ok";
    case ES_ERR_ARG: return "invalid argument";
    case ES_ERR_PIN: return "class table digest mismatch";
    case ES_ERR_RANGE: return "range outside floor/ceiling";
    case ES_ERR_FILTERS: return "bad filter file";
    case ES_ERR_CUDA: return "CUDA error";
    case ES_ERR_DEVICE_STATUS: return "device status error";
    case ES_ERR_NOMEM: return "out of memory";
    case ES_ERR_TIMEOUT: return "timeout";
    case ES_ERR_BUSY: return "busy";
  }
  return "unknown status";
}

static thread_local std::string g_open_error;   // why the last es_open on this thread failed

const char *es_last_error(const es_engine *e) { return e ? e->last_error.c_str() : g_open_error.c_str(); }

es_status es_load_filters(const char *path, uint64_t **mods, uint64_t **ress, size_t *n) {
  if (!path || !mods || !ress || !n) return ES_ERR_ARG;
  FILE *fp = fopen(path, "r");
  if (!fp) return ES_ERR_FILTERS;
  std::vector<uint64_t> m, r;
  char line[256];
  while (fgets(line, sizeof line, fp)) {
    unsigned long long a, b;
    if (sscanf(line, "FILTER %llu %llu", &a, &b) == 2) { m.push_back(a); r.push_back(b); }
  }
  fclose(fp);
  if (m.empty()) return ES_ERR_FILTERS;
  *mods = (uint64_t *)malloc(m.size() * sizeof(uint64_t));
  *ress = (uint64_t *)malloc(r.size() * sizeof(uint64_t));
  if (!*mods || !*ress) { free(*mods); free(*ress); return ES_ERR_NOMEM; }
  memcpy(*mods, m.data(), m.size() * sizeof(uint64_t));
  memcpy(*ress, r.data(), r.size() * sizeof(uint64_t));
  *n = m.size();
  return ES_OK;
}

void es_free_u64(uint64_t *p) { free(p); }

es_status es_open(const es_config *cfg, es_engine **out) {
  if (!cfg || !out) return ES_ERR_ARG;
  *out = nullptr;
  es_engine *e = new (std::nothrow) es_engine();
  if (!e) return ES_ERR_NOMEM;
  e->M = cfg->wheel_M ? cfg->wheel_M : 2042040;
  e->mmax = cfg->mmax ? cfg->mmax : 10000;
  e->sieve_p = cfg->sieve_p;
  e->device = cfg->device;
  e->flags = cfg->flags;
  if (e->flags & ES_FLAG_TEST_RHO_BUDGET) e->rho_budget = 64;
  if (e->M < 2 || e->M > 0x7FFFFFFFull) { g_open_error = "wheel modulus must be below 2^31"; delete e; return ES_ERR_ARG; }
  const std::vector<Cover> covers = gen_covers(e->mmax);
  const Wheel w = build_wheel(e->M, gen_wheel_covers(e->M), gen_ucerts(UCERT_RMAX, UCERT_UMAX));
  e->classes = w.classes;
  build_lane_index(e);
  e->wheel_pmin = w.max_pmin;
  for (const Cover &f : covers) e->cover_pmax = std::max(e->cover_pmax, f.pmin);
  e->class_fnv = fnv64_classes(e->classes);
  e->pin = class_pin(e->M);
  if (e->pin && e->class_fnv != e->pin->fnv64) {
    char buf[200];
    snprintf(buf, sizeof buf, "class table digest mismatch at M=%llu -- derived fnv64 %016llx, expected %016llx",
             e->M, e->class_fnv, e->pin->fnv64);
    g_open_error = buf;
    delete e;
    return ES_ERR_PIN;
  }
  if (e->classes.empty()) { delete e; return ES_ERR_ARG; }
  if (cfg->filter_mods) {
    if (!cfg->filter_ress || cfg->n_filters == 0) { delete e; return ES_ERR_FILTERS; }
    e->mods.assign(cfg->filter_mods, cfg->filter_mods + cfg->n_filters);
    e->ress.assign(cfg->filter_ress, cfg->filter_ress + cfg->n_filters);
  } else {
    for (const Cover &f : covers)
      if (e->M % f.mod) { e->mods.push_back(f.mod); e->ress.push_back(f.res); }
  }
  e->ncov = e->mods.size();
  if (e->sieve_p)
    for (u64 q : small_primes(e->sieve_p, e->M)) { e->mods.push_back(q); e->ress.push_back(0); }
  e->filter_fnv = fnv64_filters(e->mods, e->ress, e->ncov);
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= e->device || e->device < 0) {
    g_open_error = "no CUDA device " + std::to_string(e->device);
    delete e;
    return ES_ERR_CUDA;
  }
  if (cudaSetDevice(e->device) != cudaSuccess) { g_open_error = "cudaSetDevice failed"; delete e; return ES_ERR_CUDA; }
  cudaDeviceGetAttribute(&e->sm_count, cudaDevAttrMultiProcessorCount, e->device);
  for (Slot &sl : e->slots) {
    if (cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&sl.d_ctr, CTR_BYTES) != cudaSuccess ||
        cudaMalloc(&sl.d_status, sizeof(u32)) != cudaSuccess) {
      g_open_error = "stream or counter allocation failed";
      es_close(e);
      return ES_ERR_CUDA;
    }
    for (auto &ev : sl.ev) cudaEventCreate(&ev);
  }
  {
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    e->mem_budget = cfg->mem_budget ? cfg->mem_budget : fr / 4;   // serving admission budget
  }
  const es_status s = build_tables(e);
  if (s != ES_OK) {
    g_open_error = e->last_error;
    es_close(e);
    return s;
  }
  *out = e;
  return ES_OK;
}

es_status es_close(es_engine *e) {
  if (!e) return ES_OK;
  {
    std::lock_guard<std::mutex> lk(e->qmu);
    e->stopping = true;
  }
  e->qcv.notify_all();
  for (std::thread &t : e->workers) t.join();
  {
    // the workers finished every queued request; a poller still inside es_poll has been woken
    // and owns its request until it returns
    std::unique_lock<std::mutex> lk(e->qmu);
    e->dcv.notify_all();
    e->dcv.wait(lk, [&] { return e->pollers == 0; });
  }
  for (auto &kv : e->reqs) delete kv.second;
  cudaSetDevice(e->device);
  for (Slot &sl : e->slots) {
    if (sl.stream) cudaStreamSynchronize(sl.stream);
    drop_graph(&sl);
    cudaFree(sl.d_win); cudaFree(sl.d_cnt); cudaFree(sl.d_shortw); cudaFree(sl.d_Qm);
    cudaFree(sl.d_surv); cudaFree(sl.d_primes); cudaFree(sl.d_direct); cudaFree(sl.d_recs); cudaFree(sl.d_cand);
    cudaFree(sl.d_ctr); cudaFree(sl.d_status); cudaFree(sl.d_hdr);
    cudaFreeHost(sl.h_hdr); cudaFreeHost(sl.h_win); cudaFreeHost(sl.h_short); cudaFreeHost(sl.h_cnt);
    cudaFreeHost(sl.h_ctr); cudaFreeHost(sl.h_status); cudaFreeHost(sl.h_recs);
    for (auto &ev : sl.ev) if (ev) cudaEventDestroy(ev);
    if (sl.stream) cudaStreamDestroy(sl.stream);
  }
  cudaFree(e->d_rho); cudaFree(e->d_fdesc); cudaFree(e->d_sdist); cudaFree(e->d_tdp);
  cudaFree(e->d_K0); cudaFree(e->d_tde); cudaFree(e->d_tdi); cudaFree(e->d_tdqm);
  cudaFree(e->d_mtab); cudaFree(e->d_mdesc); cudaFree(e->d_lfil);
  delete e;
  return ES_OK;
}

es_status es_run_window(es_engine *e, uint64_t lo, uint64_t hi, es_counters *out, es_records *recs) {
  if (!e || !out) return ES_ERR_ARG;
  std::lock_guard<std::mutex> lk(e->slots[0].mu);
  cudaSetDevice(e->device);
  const auto t0 = std::chrono::steady_clock::now();
  es_window w{lo, hi};
  memset(out, 0, sizeof *out);
  if (recs) { recs->recs = nullptr; recs->n = 0; }
  const es_status st = run_windows(e, &e->slots[0], &w, 1, ES_SCHED_PERSISTENT, out, recs);
  e->slots[0].timing.host_total_ms = ms_since(t0);
  return st;
}

es_status es_run_batch(es_engine *e, const es_window *w, size_t n, int schedule, es_counters *per_window,
                       es_records *recs) {
  if (!e || (!w && n) || !per_window) return ES_ERR_ARG;
  if (schedule != ES_SCHED_PLAIN && schedule != ES_SCHED_PERSISTENT) return ES_ERR_ARG;
  std::lock_guard<std::mutex> lk(e->slots[0].mu);
  const auto t0 = std::chrono::steady_clock::now();
  cudaSetDevice(e->device);
  memset(per_window, 0, n * sizeof(es_counters));
  if (recs) { recs->recs = nullptr; recs->n = 0; }
  if (n == 0) return ES_OK;
  const es_status st = run_windows(e, &e->slots[0], w, n, schedule, per_window, recs);
  e->slots[0].timing.host_total_ms = ms_since(t0);
  return st;
}

es_status es_free_records(es_records *r) {
  if (!r) return ES_ERR_ARG;
  free(r->recs);
  r->recs = nullptr;
  r->n = 0;
  return ES_OK;
}

static char *put_u64(char *o, unsigned long long v) {
  char b[20];
  int n = 0;
  do { b[n++] = (char)('0' + (int)(v % 10)); v /= 10; } while (v);
  while (n) *o++ = b[--n];
  return o;
}

static char *put_u128(char *o, unsigned long long lo, unsigned long long hi) {
  if (!hi) return put_u64(o, lo);
  const unsigned __int128 v = ((unsigned __int128)hi << 64) | lo;
  const unsigned long long P19 = 10000000000000000000ull;
  const unsigned __int128 q = v / P19;                 // below 2^64 for every u < 2^127
  unsigned long long r = (unsigned long long)(v % P19);
  o = q >> 64 ? put_u128(o, (unsigned long long)q, (unsigned long long)(q >> 64)) : put_u64(o, (unsigned long long)q);
  char b[19];
  for (int i = 18; i >= 0; --i) { b[i] = (char)('0' + (int)(r % 10)); r /= 10; }
  memcpy(o, b, 19);
  return o + 19;
}

size_t es_format_record(const es_record *r, char *buf, size_t cap) {
  if (!r || !buf) return 0;
  char line[192];
  char *o = line;
  auto put = [&](const char *s, size_t n) { memcpy(o, s, n); o += n; };
  if (r->kind == ES_REC_RUNG) {
    put("RUNG ", 5);
    o = put_u64(o, r->p); *o++ = ' ';
    o = put_u64(o, r->a); *o++ = ' ';
    o = put_u64(o, r->b); *o++ = ' ';
    o = put_u128(o, r->c, r->d);
  } else if (r->kind == ES_REC_SOLVED) {
    put("SOLVED ", 7);
    o = put_u64(o, r->p); *o++ = ' ';
    o = put_u64(o, r->a); *o++ = ' ';
    o = put_u64(o, r->b); *o++ = ' ';
    o = put_u64(o, r->c); *o++ = ' ';
    o = put_u64(o, r->d);
  } else if (r->kind == ES_REC_SURVIVOR) {
    put("SURVIVOR ", 9);
    o = put_u64(o, r->p);
  } else {
    return 0;
  }
  *o++ = '\n';
  const size_t k = (size_t)(o - line);
  if (k >= cap) return 0;
  memcpy(buf, line, k);
  buf[k] = 0;
  return k;
}

size_t es_format_summary(const es_engine *e, uint64_t lo, uint64_t hi, const es_counters *c, char *buf, size_t cap) {
  if (!e || !c || !buf) return 0;
  const int k = snprintf(buf, cap,
                         "SUMMARY lo=%llu hi=%llu wheelM=%llu lanes=%zu mmax=%llu ucert_rmax=%u ucert_umax=%u "
                         "wheel_pmin=%llu classes_sha256=%s positions=%llu covered=%llu sieved=%llu mr=%llu "
                         "composite=%llu rung=%llu direct=%llu survivors=%llu\n",
                         (unsigned long long)lo, (unsigned long long)hi, e->M, e->classes.size(), e->mmax,
                         UCERT_RMAX, UCERT_UMAX, e->wheel_pmin, e->pin ? e->pin->sha256 : "unpinned",
                         (unsigned long long)c->positions, (unsigned long long)c->covered,
                         (unsigned long long)c->sieved, (unsigned long long)c->mr, (unsigned long long)c->composite,
                         (unsigned long long)c->rung, (unsigned long long)c->direct,
                         (unsigned long long)c->survivors);
  return (k > 0 && (size_t)k < cap) ? (size_t)k : 0;
}

es_status es_get_schedule(const es_engine *e, es_schedule *o) {
  if (!e || !o) return ES_ERR_ARG;
  *o = e->sched;
  return ES_OK;
}

es_status es_set_schedule(es_engine *e, const es_schedule *s) {
  if (!e || !s) return ES_ERR_ARG;
  if (s->short_max < 1 || s->short_max > es::SEG_SMALL)
    return fail(e, ES_ERR_ARG, "short_max must be in 1.." + std::to_string(es::SEG_SMALL));
  if (s->rung_blocks_per_sm < 1 || s->rung_blocks_per_sm > 16)
    return fail(e, ES_ERR_ARG, "rung_blocks_per_sm must be in 1..16");
  if (s->long_split > 1) return fail(e, ES_ERR_ARG, "long_split must be 0 or 1");
  for (uint32_t r : s->reserved)
    if (r) return fail(e, ES_ERR_ARG, "reserved schedule fields must be zero");
  // every slot idle while the schedule changes; their graphs hold the old launch shapes
  std::vector<std::unique_lock<std::mutex>> locks;
  for (Slot &sl : e->slots) locks.emplace_back(sl.mu);
  cudaSetDevice(e->device);
  e->sched = *s;
  for (Slot &sl : e->slots) drop_graph(&sl);
  return ES_OK;
}

es_status es_autotune(es_engine *e, const es_window *w, size_t n, int repeats, es_schedule *chosen) {
  if (!e || !w || n == 0 || repeats < 1 || repeats > 1000) return ES_ERR_ARG;
  static const uint32_t SHORT[] = {SEG_SMALL / 4, SEG_SMALL / 2, SEG_SMALL};
  static const uint32_t RUNG[] = {4, 6, 8};
  static const uint32_t SPLIT[] = {1, 0};
  const es_schedule before = e->sched;
  std::vector<es_counters> base(n), cur(n);
  es_records rbase{nullptr, 0};
  es_schedule best = before;
  double best_ms = 1e300;
  bool first = true;
  es_status st = ES_OK;
  for (uint32_t sm : SHORT) {
    for (size_t cand = 0; cand < 6; ++cand) {
      const uint32_t rb = RUNG[cand % 3], split = SPLIT[cand / 3];
      es_schedule c = before;
      c.short_max = sm;
      c.rung_blocks_per_sm = rb;
      c.long_split = split;
      if ((st = es_set_schedule(e, &c)) != ES_OK) break;
      double ms = 0;                               // mean device time of the timed runs
      for (int r = 0; r <= repeats && st == ES_OK; ++r) {
        es_records rc{nullptr, 0};
        st = es_run_batch(e, w, n, ES_SCHED_PERSISTENT, cur.data(), &rc);
        if (st != ES_OK) break;
        if (first) {                               // the first run defines the results
          base = cur;
          rbase = rc;
          first = false;
          continue;
        }
        const bool same = memcmp(cur.data(), base.data(), n * sizeof(es_counters)) == 0 && rc.n == rbase.n &&
                          (rc.n == 0 || memcmp(rc.recs, rbase.recs, rc.n * sizeof(es_record)) == 0);
        es_free_records(&rc);
        if (!same) st = fail(e, ES_ERR_DEVICE_STATUS, "autotune: a schedule changed a result");
        // run 0 warms up (graph capture). The mean, not the best, of the timed runs: stage D's
        // time varies from run to run with which walk splits the hardest cofactor first, and
        // the fastest of a few runs rewards a lucky tail rather than a better schedule.
        if (r > 0) ms += e->slots[0].timing.total_ms / repeats;
      }
      if (st != ES_OK) break;
      if (ms < best_ms) { best_ms = ms; best = c; }
    }
    if (st != ES_OK) break;
  }
  es_free_records(&rbase);
  if (st != ES_OK) { es_set_schedule(e, &before); return st; }
  st = es_set_schedule(e, &best);
  if (st == ES_OK && chosen) *chosen = best;
  return st;
}

es_status es_info(const es_engine *e, es_info_t *o) {
  if (!e || !o) return ES_ERR_ARG;
  memset(o, 0, sizeof *o);
  o->wheel_M = e->M; o->lanes = e->classes.size(); o->wheel_pmin = e->wheel_pmin;
  o->cover_pmax = e->cover_pmax; o->floor = std::max(e->wheel_pmin, e->cover_pmax);
  o->ceiling = DIRECT_PMAX; o->class_fnv64 = e->class_fnv; o->filter_fnv64 = e->filter_fnv;
  o->n_certified = e->ncov; o->n_filters = e->mods.size(); o->mmax = e->mmax;
  o->short_max_limit = es::SEG_SMALL;
  o->pinned = e->pin != nullptr;
  snprintf(o->classes_sha256, sizeof o->classes_sha256, "%s", e->pin ? e->pin->sha256 : "unpinned");
  return ES_OK;
}

es_status es_classes(const es_engine *e, uint64_t *out, size_t cap) {
  if (!e || !out) return ES_ERR_ARG;
  for (size_t i = 0; i < e->classes.size() && i < cap; ++i) out[i] = e->classes[i];
  return ES_OK;
}

es_status es_timing(const es_engine *e, es_timing_t *o) {
  if (!e || !o) return ES_ERR_ARG;
  *o = e->slots[0].timing;
  return ES_OK;
}

es_status es_is_prime_batch(es_engine *e, const uint64_t *n, size_t count, uint8_t *out) {
  if (!e || (!n && count) || (!out && count)) return ES_ERR_ARG;
  if (!count) return ES_OK;
  return probe(e, &e->slots[0], count, count * 8, n, count, {{out, count}}, [&](void *in, std::vector<void *> &o) {
    k_probe_prime<<<e->sm_count * 2, 256, 0, e->slots[0].stream>>>((const u64 *)in, count, (unsigned char *)o[0]);
  });
}

es_status es_solve_rung_batch(es_engine *e, const uint64_t *p, size_t count, es_record *out, uint8_t *found) {
  if (!e || (!p && count) || (!out && count) || (!found && count)) return ES_ERR_ARG;
  if (!count) return ES_OK;
  return probe(e, &e->slots[0], count, count * 8, p, 0, {{out, count * sizeof(es_record)}, {found, count}},
               [&](void *in, std::vector<void *> &o) {
                 k_probe_rung<<<e->sm_count * 4, RUNG_WARPS * 32, 0, e->slots[0].stream>>>((const u64 *)in, count, (RecDev *)o[0],
                                                                     (unsigned char *)o[1], e->d_tdp, e->d_tdi, e->d_tdqm,
                                                                     e->slots[0].d_status, e->rho_budget);
               });
}

es_status es_solve_direct_batch(es_engine *e, const uint64_t *p, size_t count, es_record *out, uint8_t *found) {
  if (!e || (!p && count) || (!out && count) || (!found && count)) return ES_ERR_ARG;
  if (!count) return ES_OK;
  return probe(e, &e->slots[0], count, count * 8, p, 0, {{out, count * sizeof(es_record)}, {found, count}},
               [&](void *in, std::vector<void *> &o) {
                 k_probe_direct<<<e->sm_count * 4, 32, 0, e->slots[0].stream>>>((const u64 *)in, count, (RecDev *)o[0],
                                                                       (unsigned char *)o[1], e->d_tdp, e->d_tde,
                                                                       e->slots[0].d_status);
               });
}

es_status es_factor_batch(es_engine *e, const uint64_t *n, size_t count, uint64_t *pr, uint8_t *ex, uint8_t *k) {
  if (!e || (!n && count) || (!pr && count) || (!ex && count) || (!k && count)) return ES_ERR_ARG;
  if (!count) return ES_OK;
  return probe(e, &e->slots[0], count, count * 8, n, 0, {{pr, count * MAXF * 8}, {ex, count * MAXF}, {k, count}},
               [&](void *in, std::vector<void *> &o) {
                 k_probe_factor<<<e->sm_count * 4, 128, 0, e->slots[0].stream>>>((const u64 *)in, count, (u64 *)o[0],
                                                                       (unsigned char *)o[1], (unsigned char *)o[2],
                                                                       e->d_tdp, e->d_tdi, e->slots[0].d_status,
                                                                       e->rho_budget);
               });
}

es_status es_check_records(es_engine *e, const es_record *r, size_t count, uint8_t *ok) {
  if (!e || (!r && count) || (!ok && count)) return ES_ERR_ARG;
  if (!count) return ES_OK;
  return probe(e, &e->slots[0], count, count * sizeof(es_record), r, 0, {{ok, count}},
               [&](void *in, std::vector<void *> &o) {
                 k_probe_check<<<e->sm_count * 4, 256, 0, e->slots[0].stream>>>((const RecDev *)in, count,
                                                                              (unsigned char *)o[0]);
               });
}

static es_status submit(es_engine *e, const es_window *w, size_t n, uint64_t *ticket, bool solo) {
  if (!e || !ticket || (!w && n)) return ES_ERR_ARG;
  *ticket = 0;
  const u64 floor_ = std::max(e->wheel_pmin, e->cover_pmax);
  for (size_t i = 0; i < n; ++i) {                 // refuse what a run would refuse, now
    if (w[i].hi > DIRECT_PMAX) return fail(e, ES_ERR_RANGE, "HI above the stage-E ceiling");
    if (w[i].lo <= floor_) return fail(e, ES_ERR_RANGE, "LO at or below the pmin floor");
  }
  Request *r = new (std::nothrow) Request();
  if (!r) return ES_ERR_NOMEM;
  r->w.assign(w, w + n);
  r->solo = solo;
  r->mem = request_bytes(e, w, n);
  {
    std::lock_guard<std::mutex> lk(e->qmu);
    if (e->stopping) { delete r; return ES_ERR_ARG; }
    // admission: a bounded queue, and device memory for the request's buffers within the
    // engine's budget (what is queued or in flight counts against it)
    if (e->queued_windows + n > SERVE_QUEUE_WINDOWS || e->mem_in_use + r->mem > e->mem_budget) {
      delete r;
      return fail(e, ES_ERR_BUSY, "admission refused: queue or device-memory budget full");
    }
    if (e->workers.empty())
      for (int k = 1; k <= SERVE_SLOTS; ++k) e->workers.emplace_back(serve_worker, e, k);
    r->ticket = e->next_ticket++;
    e->mem_in_use += r->mem;
    e->queued_windows += n;
    e->reqs[r->ticket] = r;
    e->queue.push_back(r);
    *ticket = r->ticket;
  }
  e->qcv.notify_one();
  return ES_OK;
}

es_status es_submit(es_engine *e, const es_window *w, size_t n, uint64_t *ticket) {
  return submit(e, w, n, ticket, false);
}

es_status es_submit_batch(es_engine *e, const es_window *w, size_t n, uint64_t *ticket) {
  return submit(e, w, n, ticket, true);
}

es_status es_poll(es_engine *e, uint64_t ticket, es_counters *per_window, es_records *recs, int timeout_ms) {
  if (!e) return ES_ERR_ARG;
  if (recs) { recs->recs = nullptr; recs->n = 0; }
  std::unique_lock<std::mutex> lk(e->qmu);
  auto it = e->reqs.find(ticket);
  if (it == e->reqs.end()) return fail(e, ES_ERR_ARG, "unknown ticket");
  Request *r = it->second;
  // One poller per ticket: a second one would read the request while the first deletes it.
  if (r->claimed) return fail(e, ES_ERR_ARG, "ticket is already being polled");
  r->claimed = true;
  ++e->pollers;
  auto ready = [&] { return r->done; };
  bool done = true;
  if (timeout_ms < 0) e->dcv.wait(lk, ready);
  else done = e->dcv.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready);
  --e->pollers;
  if (!done) {
    r->claimed = false;                  // the ticket stays valid; the caller may poll again
    e->dcv.notify_all();
    return ES_ERR_TIMEOUT;
  }
  e->reqs.erase(r->ticket);
  e->dcv.notify_all();                   // es_close may be waiting for the last poller
  lk.unlock();
  const es_status st = r->st;
  if (st == ES_OK) {
    if (per_window) memcpy(per_window, r->cnt.data(), r->cnt.size() * sizeof(es_counters));
    if (recs) {
      recs->n = r->recs.size();
      recs->recs = (es_record *)malloc(std::max<size_t>(r->recs.size(), 1) * sizeof(es_record));
      if (!recs->recs) { delete r; return ES_ERR_NOMEM; }
      memcpy(recs->recs, r->recs.data(), r->recs.size() * sizeof(es_record));
    }
  } else {
    fail(e, st, r->err);
  }
  delete r;
  return st;
}

}  // extern "C"
