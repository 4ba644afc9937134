// pa_msc_core.cuh -- device building blocks of the multi-spin-coded sweeps
// (single-CTA and cluster variants): the bitsliced neighbour adder, the
// digit-serial acceptance for 32 replicas per word, per-population parameters
// and per-bit statistics.
#pragma once

#include <climits>

#include "pa_device.cuh"

namespace pa {
namespace msc {

constexpr uint32_t kLcgA = 1664525u;     // PAisingMSC.cu:53
constexpr uint32_t kLcgC = 1013904223u;  // PAisingMSC.cu:54
constexpr uint32_t kFull = 0xffffffffu;
constexpr int kKB = 4;  // word-sites per thread decided together (native stream)
constexpr int kMaxTile = 8;                // groups per work unit of the one-CTA sweep (one warp each at least)
constexpr int kTileSmemMax = 44 * 1024;    // shared memory of a tile of more than one group

// Bitsliced count of anti-parallel neighbours (4 inputs -> 3 bit planes),
// the adder of PAisingMSC.cu:212-218.
__device__ __forceinline__ void adder4(uint32_t I1, uint32_t I2, uint32_t I3, uint32_t I4, uint32_t& s0,
                                       uint32_t& s1, uint32_t& s2) {
  const uint32_t x12 = I1 ^ I2, x34 = I3 ^ I4, a12 = I1 & I2, a34 = I3 & I4;
  s0 = x12 ^ x34;
  s1 = (x12 & x34) ^ a12 ^ a34;
  s2 = a12 & a34;
}

// Per-replica-bit sums over the words of a warp, for the energy epilogue.
// Each lane adds its words' bond counts (0..4 per word, as adder4's planes
// s0 + 2 s1 + 4 s2) and spin bits into bitsliced counters -- bit k of plane
// l holds bit l of the lane's running count for replica bit k -- at a few
// logic operations per word instead of a warp vote per replica bit.  At the
// end each plane is transposed across the warp (bit i of lane k <- bit k of
// lane i) and counted, so lane k receives bit k's sums over the warp.  Eight
// and seven planes hold the counts of up to 63 words per lane.
struct BitCounters {
  uint32_t e[8], m[7];
  __device__ __forceinline__ void reset() {
#pragma unroll
    for (int l = 0; l < 8; ++l) e[l] = 0u;
#pragma unroll
    for (int l = 0; l < 7; ++l) m[l] = 0u;
  }
  // c += x << at, bit by bit (ripple of half adders)
  template <int NL>
  __device__ __forceinline__ static void ripple(uint32_t (&c)[NL], int at, uint32_t x) {
#pragma unroll
    for (int l = 0; l < NL; ++l)
      if (l >= at) {
        const uint32_t t = c[l] & x;
        c[l] ^= x;
        x = t;
      }
  }
  __device__ __forceinline__ void add(uint32_t s0, uint32_t s1, uint32_t s2, uint32_t sA, uint32_t sB) {
    ripple(e, 0, s0);
    ripple(e, 1, s1);
    ripple(e, 2, s2);
    ripple(m, 0, sA ^ sB);
    ripple(m, 1, sA & sB);
  }
  __device__ __forceinline__ static uint32_t transpose(uint32_t x, int lane) {
#pragma unroll
    for (int j = 16; j >= 1; j >>= 1) {
      const uint32_t lo = j == 16 ? 0x0000FFFFu : j == 8 ? 0x00FF00FFu : j == 4 ? 0x0F0F0F0Fu
                                                 : j == 2 ? 0x33333333u : 0x55555555u;  // bit positions b & j == 0
      const uint32_t y = __shfl_xor_sync(kFull, x, j);
      x = (lane & j) ? (x & ~lo) | ((y >> j) & lo) : (x & lo) | ((y & lo) << j);
    }
    return x;
  }
  // whole warp: lane k gets the sums of replica bit k
  __device__ __forceinline__ void totals(int lane, int& cE, int& cM) const {
    cE = 0;
    cM = 0;
#pragma unroll
    for (int l = 0; l < 8; ++l) cE += __popc(transpose(e[l], lane)) << l;
#pragma unroll
    for (int l = 0; l < 7; ++l) cM += __popc(transpose(m[l], lane)) << l;
  }
};

// The two masks the acceptance needs from a word's four neighbour words:
// odd = an odd number of anti-parallel neighbours (among undecided bits: one,
// threshold T4), ge2 = two or more (dE <= 0: flipped outright) -- adder4's s0
// and s1 | s2, in fewer logic operations: the XOR of two neighbours does not
// depend on the spin itself, and "two or more" is a pair within either half
// or one in each.
__device__ __forceinline__ void count_masks(uint32_t s, uint32_t n1, uint32_t n2, uint32_t n3, uint32_t n4,
                                            uint32_t& odd, uint32_t& ge2) {
  const uint32_t x12 = n1 ^ n2, x34 = n3 ^ n4;
  const uint32_t a12 = (s ^ n1) & (s ^ n2), a34 = (s ^ n3) & (s ^ n4);
  odd = x12 ^ x34;
  ge2 = a12 | a34 | (x12 & x34);
}

// One binary digit of the comparison U < T/2^32 done for 32 bits at once:
// U's digit j is bit i of the random word u for replica bit i, T's digit j
// is selected per bit from T4 (bits in s0: one anti-parallel neighbour,
// dE = 4) or T8 (no anti-parallel neighbour, dE = 8).  dg = digit_table(j)
// gives that selection as one multiply-add, p = s0 * dg.x + dg.y (see
// digit_table).  Bits decided at this digit leave `und` (a subtraction, since
// they are a subset of it); those decided "less" enter `lt`.  The
// multiply-add and the subtraction issue on the FMA pipe, leaving the ALU
// pipe -- the sweep's busiest -- two logic operations per digit.
__device__ __forceinline__ void digit_step(uint32_t u, uint32_t s0, uint2 dg, uint32_t& und, uint32_t& lt) {
  const uint32_t p = s0 * dg.x + dg.y;
  const uint32_t dec = und & (p ^ u);
  lt |= dec & p;
  und -= dec;
}

// Digit j of the thresholds T4, T8 as (m, c) with s0 * m + c = the bits'
// threshold digits: T4's digit where s0 is set, T8's elsewhere.  With D = all
// ones iff the digit is 1: both digits equal -> (0, D8); T4's 1, T8's 0 ->
// (1, 0) = s0; T4's 0, T8's 1 -> (-1, ~0) = ~s0.
__host__ __device__ inline uint2 digit_table(uint32_t T4, uint32_t T8, int j) {
  const uint32_t b4 = (T4 >> (31 - j)) & 1u, b8 = (T8 >> (31 - j)) & 1u;
  return make_uint2(b4 == b8 ? 0u : b4 ? 1u : 0xFFFFFFFFu, 0u - b8);
}

// The last undecided bits of a comparison word: their first 8 digits equal
// T's, so U < T/2^32 is decided by the remaining 24 digits at once,
// U mod 2^24 < T mod 2^24, with one fresh 32-bit word w per bit (its top 24
// bits are U's remaining digits): w < (T mod 2^24) * 2^8, compared against
// t4 = T4 << 8 and t8 = T8 << 8.  Takes the lowest undecided bit; a no-op
// when none is left.
__device__ __forceinline__ void finish_bit(uint32_t w, uint32_t am, uint32_t t4, uint32_t t8, uint32_t& und,
                                           uint32_t& lt) {
  const uint32_t b = und & (0u - und);
  const uint32_t t = (am & b) ? t4 : t8;
  // b is a bit of und and not yet of lt: the updates are additions, which
  // the FMA pipe can take (the sweep's logic operations keep the ALU pipe
  // the busier one)
  lt += w < t ? b : 0u;
  und -= b;
}

// Tag of the words that finish single bits (finish_bit): the sweep's tag with
// bit 29 flipped ('M' -> 'm', 'S' -> 's'), a stream of its own.
constexpr uint32_t kFinishTagFlip = 0x20u << 24;

// Remaining digits (from digit 4 on) of one 32-bit comparison word: digits
// 4..7 of every bit from one Philox block (counter (c0, c1 | sub, step,
// tag)); the few bits still undecided after them (1/16 of those entering)
// are finished one at a time by finish_bit, four per Philox block (counter
// (c0, c1 | (fsub + k), step, tag ^ kFinishTagFlip), k = 0..7, enough for all
// 32 bits).  Returns the bits decided "less".
template <class Keys>
__device__ __forceinline__ uint32_t finish_digits(uint32_t und, uint32_t am, uint32_t c0, uint32_t c1, uint32_t sub,
                                                  uint32_t fsub, uint32_t step, uint32_t tag, const Keys& K,
                                                  const uint2* dig, uint32_t T4, uint32_t T8) {
  // no vote first: some lane of the warp nearly always has undecided bits
  // here (and the overflow path only calls when one has); a lane without
  // them is left unchanged by every step below
  uint32_t lt = 0;
  {
    const U4 r = philox10k(c0, c1 | sub, step, tag, K);
    digit_step(r.x, am, dig[4], und, lt);
    digit_step(r.y, am, dig[5], und, lt);
    digit_step(r.z, am, dig[6], und, lt);
    digit_step(r.w, am, dig[7], und, lt);
  }
  const uint32_t t4 = T4 << 8, t8 = T8 << 8, ftag = tag ^ kFinishTagFlip;
  // the first block without a vote either: nearly every warp has a lane with
  // a bit left after digit 7
#pragma unroll 1
  for (uint32_t k = 0; k < 8u; ++k) {
    if (k > 0 && !__any_sync(kFull, und != 0u)) break;
    const U4 r = philox10k(c0, c1 | (fsub + k), step, ftag, K);
    finish_bit(r.x, am, t4, t8, und, lt);
    finish_bit(r.y, am, t4, t8, und, lt);
    finish_bit(r.z, am, t4, t8, und, lt);
    finish_bit(r.w, am, t4, t8, und, lt);
  }
  return lt;
}

// Exact Metropolis decisions U < T/2^32 for kKB word-sites of one thread.
// Head: digits 0..3 of every site come from the site's own Philox block;
// after them only ~1/16 of the bits are undecided.  Tail: those sparse bits
// of the kKB sites are merged into one word, site k's masks rotated by rot_k
// so that every (site, replica) pair gets its own bit position -- hence its
// own fresh digits -- and the remaining digits are drawn once for all sites.
// A site whose bits find no free rotation is finished on its own.
//   a[k]   : bits with one anti-parallel neighbour (threshold T4), else T8
//   und[k] : bits needing a random decision (consumed)
//   acc[k] : accepted bits (in: outright accepts; out: all accepts)
//   nvalid : block-uniform count of the leading slots that hold sites; the
//            other slots have und = 0 and draw nothing
//   K      : PhiloxKeys or PhiloxKeysWide (the same stream, two code forms)
template <class Keys>
__device__ __forceinline__ void accept_native(const uint32_t (&a)[kKB], uint32_t (&und)[kKB], uint32_t (&acc)[kKB],
                                              const uint32_t (&site)[kKB], uint32_t chain_c0, uint32_t c1,
                                              uint32_t step, uint32_t tag, const Keys& K, const uint2* dig,
                                              int nvalid, uint32_t T4, uint32_t T8) {
  // independent Philox chains of the kKB sites, interleaved by the compiler
  const uint2 d0 = dig[0], d1 = dig[1], d2 = dig[2], d3 = dig[3];
  auto head = [&](int k) {
    const U4 r = philox10k(site[k], c1, step, tag, K);
    digit_step(r.x, a[k], d0, und[k], acc[k]);
    digit_step(r.y, a[k], d1, und[k], acc[k]);
    digit_step(r.z, a[k], d2, und[k], acc[k]);
    digit_step(r.w, a[k], d3, und[k], acc[k]);
  };
  if (nvalid >= kKB) {
#pragma unroll
    for (int k = 0; k < kKB; ++k) head(k);
  } else {
#pragma unroll
    for (int k = 0; k < kKB; ++k)
      if (k < nvalid) head(k);
  }
  uint32_t m = und[0], am = a[0] & und[0];
  uint32_t rot[kKB];
  rot[0] = 0;
  uint32_t ovf = 0;
#pragma unroll
  for (int k = 1; k < kKB; ++k) {
    uint32_t r = 0;
    while (r < 32u && (m & __funnelshift_l(und[k], und[k], r))) ++r;
    rot[k] = r;
    if (r < 32u) {  // disjoint from the bits merged so far: additions, on the FMA pipe
      m += __funnelshift_l(und[k], und[k], r);
      am += __funnelshift_l(a[k] & und[k], a[k] & und[k], r);
    } else {
      ovf |= 1u << k;
    }
  }
  const uint32_t lt = finish_digits(m, am, chain_c0, c1, 1u, 0u, step, tag, K, dig, T4, T8);
  acc[0] |= lt & und[0];
#pragma unroll
  for (int k = 1; k < kKB; ++k)
    if (!(ovf >> k & 1u)) acc[k] |= __funnelshift_r(lt, lt, rot[k]) & und[k];
  if (__any_sync(kFull, ovf != 0u)) {  // rare: one vote for the three sites
#pragma unroll
    for (int k = 1; k < kKB; ++k)
      if (__any_sync(kFull, ovf >> k & 1u))
        acc[k] |= finish_digits((ovf >> k & 1u) ? und[k] : 0u, a[k] & und[k], site[k], c1, 8u, 8u, step, tag, K,
                                dig, T4, T8);
  }
}

// One-group work units keep each sublattice in shared memory as L + 2 rows of
// Wr words (row -1 and row L are periodic copies); sublattice B's block
// starts at this word offset (A's block rounded up to 16 bytes).
__host__ __device__ inline int msc_halo_block(int L, int Wr) { return ((L + 2) * Wr + 3) & ~3; }

// Per-population parameters of the group a CTA is annealing.  They live in
// shared memory and are read where used, which keeps the hot loops' register
// footprint independent of how many populations the batch holds.
struct UnitParams {
  int L, N, h, Wr, rpp, npass, kconst, step, sweeps, nbatch;
  int G, rg;                    // groups per tile, groups in the population
  int sb;                       // one-group units: word offset of sublattice B's block in shared memory
  uint32_t invL, invWr, invH4;  // reciprocals (recip32) of L, Wr and h/4
  uint32_t tag, T4, T8;
  unsigned long long seed, iseq;
  uint32_t* words;
  const uint8_t* act;
  int32_t* E;
  int32_t* M;
};

// Statistics of the groups a CTA annealed for one population, accumulated in
// shared memory by lane k of warp 0 for replica bit k (registers stay free
// for the sweep); flushed to the population when the CTA moves on.
struct BitStats {
  long long sE[kMsb], sE2[kMsb], sM[kMsb], sM2[kMsb];
  unsigned long long m4lo[kMsb], m4hi[kMsb];
  int emin[kMsb];
  __device__ void reset(int k) {
    sE[k] = sE2[k] = sM[k] = sM2[k] = 0;
    m4lo[k] = m4hi[k] = 0;
    emin[k] = INT_MAX;
  }
  __device__ void add(int k, int E, int Mg) {
    const long long am = Mg < 0 ? -(long long)Mg : (long long)Mg;
    sE[k] += E;
    sE2[k] += (long long)E * E;
    sM[k] += am;
    sM2[k] += am * am;
    unsigned long long lo, hi;
    m4_of(Mg, lo, hi);
    U128 m{m4lo[k], m4hi[k]};
    u128_add(m, lo, hi);
    m4lo[k] = m.lo;
    m4hi[k] = m.hi;
    emin[k] = E < emin[k] ? E : emin[k];
  }
  // warp 0 only, lane k = bit k
  __device__ void flush(PopDev* st, int k) {
    const long long e = warp_sum(sE[k]), e2 = warp_sum(sE2[k]), m = warp_sum(sM[k]), m2 = warp_sum(sM2[k]);
    const int mn = warp_min(emin[k]);
    U128 q{m4lo[k], m4hi[k]};
    for (int o = 16; o > 0; o >>= 1) {  // 128-bit sum across the warp, carries into hi
      const unsigned long long lo = __shfl_xor_sync(kFull, q.lo, o);
      const unsigned long long hi = __shfl_xor_sync(kFull, q.hi, o);
      u128_add(q, lo, hi);
    }
    if (k == 0 && mn != INT_MAX) {
      atomicAdd((unsigned long long*)&st->sE, (unsigned long long)e);
      atomicAdd((unsigned long long*)&st->sE2, (unsigned long long)e2);
      atomicAdd((unsigned long long*)&st->sM, (unsigned long long)m);
      atomicAdd((unsigned long long*)&st->sM2, (unsigned long long)m2);
      u128_atomic_add(&st->sM4lo, &st->sM4hi, q.lo, q.hi);
      atomicMin(&st->Emin_acc, mn);
    }
    reset(k);
  }
};

}  // namespace msc
}  // namespace pa
