// pa_ssc_bits.cu -- single-spin-coded populations swept on bit planes
// (native stream).
//
// The population stays in the SSC layout in HBM (one int8 +-1 per site,
// sublattice A then B, site (x, y) at idx = y*L/2 + x/2, PAisingSSC.cu:169).
// A CTA loads a tile of replicas and packs every sublattice row (S = L/2
// sites) into bits, 1 == +1: "multi-site coding".  A row takes Wq words of
// `seg` sites each (seg a multiple of 4, at most 32); when a row fits one
// word, floor(32/seg) rows of different replicas share it as segments (L=16:
// 4 replicas x 8 sites, L=32: 2 x 16, L=48: one 24-site segment).  In a
// checkerboard half-sweep the sites of one sublattice are independent, so a
// word is updated at once: its four neighbour words are the other
// sublattice's rows y-1, y, y+1 and row y shifted by one site towards x-1 or
// x+1 by row parity (PAisingSSC.cu:170,182) -- periodically inside each
// segment, or across the row's words -- their anti-parallel counts come from
// the bitsliced adder, and the decisions from the digit-serial acceptance of
// the multi-spin-coded sweep (accept_native): each site flips with
// probability exactly min(1, T/2^32), T = ceil(2^32 e^{-beta dE}), the
// thresholds of the int8 sweep.  Bits outside the segments stay 0.  The
// energy and magnetisation of each replica are population counts of its
// segments.  The tile is unpacked and written back once per temperature.
//
// Work per tile and half-sweep: about 1024 words, four per thread, decided
// together (kKB = 4).  L = 64 and 128 (rows of one or two full words) have a
// form of their own (half_full): a thread takes four consecutive rows of one
// replica's word column, and the word groups carry periodic copies of rows -1
// and L, padded to a bank-conflict-free stride (full_stride).
#include <type_traits>

#include "pa_kernels.h"
#include "pa_msc_core.cuh"

namespace pa {

using namespace msc;

namespace {

constexpr uint32_t kLsb4 = 0x01010101u;
constexpr int kTileWords = 1024;    // words of one plane of a tile (4 per thread)
constexpr int kMaxBitsTile = 256;   // replicas per tile (one counter each)

// bits j of the 4 bytes of w (+1 -> 1, -1 -> 0), j = byte index
__device__ __forceinline__ uint32_t pack4(uint32_t w) {
  const uint32_t plus = ~(w >> 1) & kLsb4;  // +1 = 0x01, -1 = 0xFF
  return (plus * 0x01020408u) >> 24;        // byte j's bit 0 to bit j
}
// 4 bits to 4 bytes: bit j set -> +1 (0x01), clear -> -1 (0xFF)
__device__ __forceinline__ uint32_t unpack4(uint32_t n) {
  const uint32_t ones = (n * 0x00204081u) & kLsb4;
  return 0xFFFFFFFFu ^ (ones * 0xFEu);
}
// seg int8 spins at p (4-byte aligned) <-> bits 0..seg-1
__device__ __forceinline__ uint32_t pack_seg(const uint8_t* p, int seg) {
  uint32_t b = 0;
  for (int i = 0; i < seg; i += 4) b |= pack4(*reinterpret_cast<const uint32_t*>(p + i)) << i;
  return b;
}
__device__ __forceinline__ void unpack_seg(uint32_t b, uint8_t* p, int seg) {
  for (int i = 0; i < seg; i += 4) *reinterpret_cast<uint32_t*>(p + i) = unpack4((b >> i) & 0xFu);
}

// Parameters of the population a CTA is sweeping (shared memory).
struct BitsParams {
  int L, N, h, S;          // lattice side, sites, sites per sublattice, sites per sublattice row
  int Wq, seg, segs, wpp;  // words per row, sites per segment, segments per word, words per plane of a word group
  int GW, G, R;            // word groups (of segs replicas) per tile, replicas per tile, replicas
  int gs, r0;              // words per word group in shared memory, offset of its row 0 (see full_stride)
  uint32_t invWpp, invWq;  // ceil(2^32 / wpp), ceil(2^32 / Wq) (Wq > 1)
  uint32_t M0, ML, V;      // first site of every segment, last site of every segment, all segment bits
  int step, sweeps;
  uint32_t tag, T4, T8;
  uint8_t* spins;
  int32_t* E;
  int32_t* M;
};

// L = 64 and 128 (rows of Wq = 1 or 2 full 32-site words, a replica per word
// group): a word group's rows are a block of full_stride(Wq) words in shared
// memory, row y at (y + 1) Wq and periodic copies of rows L-1 and 0 before
// and after, so the sweep reads vertical neighbours without wrapping.  The
// stride is Wq modulo 32 so that the 32 lanes of a warp -- 4 groups x 32/(4 Wq)
// blocks of 4 rows x Wq words -- hit 32 different banks.
__host__ __device__ constexpr bool full_rows(int Wq, int seg) { return seg == 32 && (Wq == 1 || Wq == 2); }
__host__ __device__ constexpr int full_stride(int Wq) {
  return ((64 * Wq + 2) * Wq + 31 - Wq) / 32 * 32 + Wq;  // >= (L + 2) Wq, = Wq mod 32
}
static_assert(full_stride(1) == 97 && full_stride(2) == 290, "strides");

// Row layout of L: Wq words of seg sites, segs = segments per word.
__host__ __device__ inline bool bits_layout(int L, int* Wq, int* seg, int* segs) {
  if (L < 8 || L % 8 != 0 || L > 256) return false;
  const int S = L / 2;
  for (int w = (S + 31) / 32; w <= 8; ++w)
    if (S % w == 0 && (S / w) % 4 == 0) {
      *Wq = w;
      *seg = S / w;
      *segs = w == 1 ? 32 / *seg : 1;
      return true;
    }
  return false;
}

__device__ __forceinline__ uint32_t recip32_dev(uint32_t d) {
  return (uint32_t)((0x100000000ull + d - 1) / d);
}

// word `it` of a plane of the tile -> word group g, word wr of the group,
// row y, word c of the row
__device__ __forceinline__ void bits_split(const BitsParams& P, int it, int& g, int& wr, int& y, int& c) {
  g = (int)__umulhi((uint32_t)it, P.invWpp);
  wr = it - g * P.wpp;
  y = P.Wq == 1 ? wr : (int)__umulhi((uint32_t)wr, P.invWq);
  c = wr - y * P.Wq;
}

// the other horizontal neighbour of the sites of word c of row `row` (word
// offset) of plane o: sites i-1 (left) or i+1, periodic inside the row
__device__ __forceinline__ uint32_t bits_side(const BitsParams& P, const uint32_t* o, int row, int c, uint32_t ctr,
                                              bool left) {
  const int Wq = P.Wq, seg = P.seg;
  if (Wq == 1)
    return left ? (((ctr << 1) & ~P.M0) | ((ctr >> (seg - 1)) & P.M0)) & P.V
                : (((ctr >> 1) & ~P.ML) | ((ctr << (seg - 1)) & P.ML)) & P.V;
  if (left) return ((ctr << 1) | (o[row + (c == 0 ? Wq - 1 : c - 1)] >> (seg - 1))) & P.V;
  return (ctr >> 1) | ((o[row + (c + 1 == Wq ? 0 : c + 1)] & 1u) << (seg - 1));
}

// replicas of tile ti present, and the words of one plane they occupy
__device__ __forceinline__ int bits_present(const BitsParams& P, int ti) { return min(P.G, P.R - ti * P.G); }
__device__ __forceinline__ int bits_items(const BitsParams& P, int ti) {
  return (bits_present(P, ti) + P.segs - 1) / P.segs * P.wpp;
}

// int8 replicas of tile ti -> bit planes (to_smem), or back
__device__ __noinline__ void bits_move(const BitsParams& P, uint32_t* pl, int ti, bool to_smem) {
  const int r0 = ti * P.G, gc = bits_present(P, ti), items = bits_items(P, ti);
  for (int it = threadIdx.x; it < 2 * items; it += blockDim.x) {
    const int X = it >= items ? 1 : 0;
    int g, wr, y, c;
    bits_split(P, it - X * items, g, wr, y, c);
    uint32_t* word = pl + (X * P.GW + g) * P.gs + P.r0 + wr;
    uint32_t w = to_smem ? 0u : *word;
    for (int j = 0; j < P.segs; ++j) {
      const int rep = g * P.segs + j;
      if (rep >= gc) break;
      uint8_t* sp = P.spins + (size_t)(r0 + rep) * P.N + X * P.h + y * P.S + c * P.seg;
      if (to_smem) w |= pack_seg(sp, P.seg) << (j * P.seg);
      else unpack_seg(w >> (j * P.seg), sp, P.seg);
    }
    if (to_smem) *word = w;
  }
  if (to_smem && P.r0) {  // periodic copies of the first and last rows
    __syncthreads();
    const int ng = items / P.wpp, L = P.L, Wq = P.Wq;
    for (int it = threadIdx.x; it < 4 * ng * Wq; it += blockDim.x) {
      const int c = it % Wq, r = it / Wq, X = r >= 2 * ng ? 1 : 0, q = r - X * 2 * ng, g = q >> 1, top = q & 1;
      uint32_t* blk = pl + (X * P.GW + g) * P.gs;
      if (top) blk[c] = blk[L * Wq + c];                 // row -1 = row L-1
      else blk[(L + 1) * Wq + c] = blk[Wq + c];          // row L = row 0
    }
  }
}

// anti-parallel bonds (each seen from its A end) and +1 sites of every
// replica of tile ti
__device__ __noinline__ void bits_count(const BitsParams& P, const uint32_t* pl, int ti, int* s_anti, int* s_plus) {
  const int gc = bits_present(P, ti), items = bits_items(P, ti), L = P.L, Wq = P.Wq;
  for (int it = threadIdx.x; it < items; it += blockDim.x) {
    int g, wr, y, c;
    bits_split(P, it, g, wr, y, c);
    const uint32_t* A = pl + g * P.gs + P.r0;
    const uint32_t* B = pl + (P.GW + g) * P.gs + P.r0;
    const uint32_t a = A[wr], ctr = B[wr];
    const uint32_t up = B[(y == 0 ? L - 1 : y - 1) * Wq + c], dn = B[(y + 1 == L ? 0 : y + 1) * Wq + c];
    const uint32_t side = bits_side(P, B, y * Wq, c, ctr, (y & 1) == 0);
    const uint32_t x1 = a ^ ctr, x2 = a ^ side, x3 = a ^ up, x4 = a ^ dn;
    if (P.segs == 1) {
      atomicAdd(&s_anti[g], __popc(x1) + __popc(x2) + __popc(x3) + __popc(x4));
      atomicAdd(&s_plus[g], __popc(a) + __popc(ctr));
    } else {
      const uint32_t m = (1u << P.seg) - 1u;  // seg <= 16 here
      for (int j = 0; j < P.segs; ++j) {
        const int rep = g * P.segs + j;
        if (rep >= gc) break;
        const uint32_t mj = m << (j * P.seg);
        atomicAdd(&s_anti[rep], __popc(x1 & mj) + __popc(x2 & mj) + __popc(x3 & mj) + __popc(x4 & mj));
        atomicAdd(&s_plus[rep], __popc(a & mj) + __popc(ctr & mj));
      }
    }
  }
}

}  // namespace

bool ssc_bits_geom(int L, SweepGeom* g, int tile, long long replicas, int slots) {
  int Wq, seg, segs;
  if (!bits_layout(L, &Wq, &seg, &segs)) return false;
  const int wpp = L * Wq;
  int GWmax = kTileWords / wpp;
  if (GWmax < 1) GWmax = 1;
  if (GWmax * segs > kMaxBitsTile) GWmax = kMaxBitsTile / segs;
  int GW = GWmax;
  if (tile > 0) {  // replicas per tile asked for: a power-of-two fraction of the largest tile
    bool ok = false;
    for (int w = GWmax; w >= 1 && !ok; w /= 2) ok = w * segs == tile;
    if (!ok) return false;
    GW = tile / segs;
  } else if (replicas > 0 && slots > 0) {
    // the largest tile that still leaves a tile for every resident CTA:
    // smaller tiles give a thread fewer than four words and so lose the
    // acceptance's sharing of undecided bits across them (at a full GPU L=64
    // tiles of 8 replicas ran 1.7x slower than 16); fewer tiles than CTAs
    // leave SMs idle (one L=16 population of 20000: 256 replicas per tile
    // 370 attempts/ns, 32 per tile 503)
    GW = 1;
    for (int w = GWmax; w >= 1; w /= 2)
      if ((replicas + (long long)w * segs - 1) / ((long long)w * segs) >= slots) {
        GW = w;
        break;
      }
  }
  g->L = L;
  g->N = L * L;
  g->half = g->N / 2;
  g->Wr = Wq;
  g->seg = seg;
  g->G = GW * segs;  // replicas per tile
  g->T = kSweepThreads;
  g->rpp = 0;
  g->npass = (GW * wpp + kSweepThreads - 1) / kSweepThreads;  // words per thread per half-sweep
  g->kconst = 0;
  g->smem = GW * 2 * (full_rows(Wq, seg) ? full_stride(Wq) : wpp) * 4;
  return true;
}

double ssc_bits_fill(int L) {
  int Wq, seg, segs;
  if (!bits_layout(L, &Wq, &seg, &segs)) return 0.0;
  return (double)(L / 2) * (Wq == 1 ? segs : 1) / (32.0 * Wq);
}

__global__ void __launch_bounds__(kSweepThreads, 4)
    ssc_sweep_bits_kernel(BatchDev* b, int energy_only, const __grid_constant__ PhiloxKeysWide keys) {
  extern __shared__ __align__(16) uint32_t pl[];  // [X][word group][y][c]: plane X, row y, word c
  __shared__ int s_unit, s_pop;
  __shared__ uint2 s_dig[kMsb];
  __shared__ int s_anti[kMaxBitsTile], s_plus[kMaxBitsTile];
  __shared__ BitsParams P;
  __shared__ BitStats stats;  // lane k accumulates the replicas k, k+32, ... of its tiles

  static_assert(kMaxBitsTile == kSweepThreads, "one counter per thread to clear");
  const int tid = threadIdx.x;
  const int total = b->unit_prefix[b->npop];
  int cur = -1;
  if (tid < kMsb) stats.reset(tid);

  for (;;) {
    __syncthreads();
    if (tid == 0) {
      const int u = (int)atomicAdd(&b->work_next, 1u);
      int loc = 0;
      const int p = u < total ? queue_pop(b, u, &loc) : -1;
      s_pop = p;
      s_unit = loc;
      if (p >= 0 && p != cur) {
        const PopDev* st = b->pops + p;
        P.L = st->L; P.N = st->N; P.h = st->N >> 1; P.S = st->L >> 1;
        P.Wq = st->Wr; P.seg = st->seg; P.segs = P.Wq == 1 ? 32 / P.seg : 1;
        P.wpp = P.L * P.Wq;
        P.r0 = full_rows(P.Wq, P.seg) ? P.Wq : 0;
        P.gs = P.r0 ? full_stride(P.Wq) : P.wpp;
        P.G = st->gpt;
        P.GW = P.G / P.segs;
        P.R = st->R_cur;
        P.invWpp = recip32_dev((uint32_t)P.wpp);
        P.invWq = P.Wq > 1 ? recip32_dev((uint32_t)P.Wq) : 0u;
        uint32_t m0 = 0;
        for (int j = 0; j < P.segs; ++j) m0 |= 1u << (j * P.seg);
        P.M0 = m0;
        P.ML = m0 << (P.seg - 1);
        P.V = P.segs * P.seg == 32 ? 0xffffffffu : (1u << (P.segs * P.seg)) - 1u;
        P.step = (int)native_step_word(st);
        P.sweeps = energy_only ? 0 : st->sweeps;
        P.tag = kTagSscSweep | (uint32_t)st->pop_id;
        P.T4 = st->thr[(size_t)st->step * kThrPerStep + 10];
        P.T8 = st->thr[(size_t)st->step * kThrPerStep + 11];
        P.spins = (uint8_t*)st->spins[st->parity];
        P.E = st->E;
        P.M = st->M;
      }
    }
    s_anti[tid] = 0;
    s_plus[tid] = 0;
    __syncthreads();
    const int p = s_pop, ti = s_unit;
    if (p < 0) break;
    if (p != cur) {  // block-uniform
      if (tid < kMsb && cur >= 0) stats.flush(b->pops + cur, tid);
      cur = p;
      if (tid < kMsb) {
        s_dig[tid] = digit_table(P.T4, P.T8, tid);
      }
    }
    bits_move(P, pl, ti, true);
    __syncthreads();

    // one half-sweep over the words of plane `self` (every layout but L = 64's)
    {
    const int L = P.L, Wq = P.Wq, seg = P.seg, wpp = P.wpp, GW = P.GW, items = bits_items(P, ti);
    auto half_sweep = [&](uint32_t* self, const uint32_t* oth, int hf, uint32_t c1) {
#pragma unroll 1
      for (int q0 = 0; q0 * kSweepThreads < items; q0 += kKB) {
        uint32_t av[kKB], un[kKB], ac[kKB], site[kKB];
        uint32_t vm = 0;
#pragma unroll
        for (int k = 0; k < kKB; ++k) {
          const int it = tid + (q0 + k) * kSweepThreads;
          const bool valid = it < items;
          const int itc = valid ? it : 0;
          const int g = (int)__umulhi((uint32_t)itc, P.invWpp), wr = itc - g * wpp;
          int y = wr, c = 0;
          if (Wq > 1) {
            y = (int)__umulhi((uint32_t)wr, P.invWq);
            c = wr - y * Wq;
          }
          const int base = g * wpp;
          const int rowu = (y == 0 ? L - 1 : y - 1) * Wq, rowd = (y + 1 == L ? 0 : y + 1) * Wq;
          const uint32_t s = self[base + wr];
          const uint32_t ctr = oth[base + wr], up = oth[base + rowu + c], dn = oth[base + rowd + c];
          const bool left = (hf == 0) == ((y & 1) == 0);
          const uint32_t side = bits_side(P, oth + base, y * Wq, c, ctr, left);
          uint32_t odd, ge2;
          count_masks(s, ctr, side, up, dn, odd, ge2);
          const uint32_t v = P.V;  // the bits of the word's segments
          av[k] = odd;
          ac[k] = ge2 & v;
          un[k] = valid ? v - ac[k] : 0u;  // = ~ge2 & v, on the FMA pipe
          vm |= valid ? 1u << k : 0u;
          site[k] = (uint32_t)(ti * GW + g) * (uint32_t)wpp + (uint32_t)wr;  // word number in the population
        }
        const uint32_t chain = ((uint32_t)ti * blockDim.x + (uint32_t)tid) * 8u + (uint32_t)(q0 / kKB);
        // slots holding words lead (it grows with k): no Philox work for the rest
        accept_native(av, un, ac, site, chain, c1, (uint32_t)P.step, P.tag, keys, s_dig, __popc(vm), P.T4, P.T8);
#pragma unroll
        for (int k = 0; k < kKB; ++k)
          if (vm >> k & 1u) self[site[k] - (uint32_t)(ti * GW) * (uint32_t)wpp] ^= ac[k];
      }
    };
    // L = 64, 128 (rows of kWq full words): lane = (gl * kRL + rl) * kWq + c of
    // warp w takes the 4 consecutive rows 4 rb .. 4 rb + 3, rb = kRL (w / (kGW/4))
    // + rl, of word column c of word group 4 (w % (kGW/4)) + gl, so the 4 words
    // share the other plane's rows around them (6 loads for 4 words, plus the
    // row's other word for the horizontal neighbour when kWq = 2); one batch
    // per thread and half-sweep
    auto half_full = [&](auto wq_c, uint32_t* self, const uint32_t* oth, int hf, uint32_t c1) {
      constexpr int kWq = decltype(wq_c)::value, kL = 64 * kWq, kGW = 1024 / (kL * kWq), kRL = 8 / kWq;
      constexpr int kS = full_stride(kWq);
      static_assert(kGW % 4 == 0 && (kGW / 4) * (kL / 4 / kRL) * 32 == kSweepThreads, "one batch per thread");
      const int lane = tid & 31, w = tid >> 5;
      const int c = lane % kWq, gl = (lane / kWq) / kRL, rl = (lane / kWq) % kRL;
      const int g = 4 * (w % (kGW / 4)) + gl, y0 = 4 * (kRL * (w / (kGW / 4)) + rl);
      const bool valid = g < items / wpp;  // word groups present in this tile
      const int gc = valid ? g : 0;
      const uint32_t* ob = oth + gc * kS + c;  // word c of row y of the other plane at ob[(y + 1) kWq]
      uint32_t* sb = self + gc * kS + kWq + c;  // and of this plane at sb[y kWq]
      uint32_t o[kKB + 2];
#pragma unroll
      for (int j = 0; j < kKB + 2; ++j) o[j] = ob[(y0 + j) * kWq];  // rows y0-1 .. y0+4
      uint32_t av[kKB], un[kKB], ac[kKB], site[kKB];
#pragma unroll
      for (int k = 0; k < kKB; ++k) {
        const uint32_t s = sb[(y0 + k) * kWq], ctr = o[k + 1];
        // y0 is even: the other horizontal neighbour is x-1 for A on even rows
        // and B on odd rows (PAisingSSC.cu:170,182): the word shifted by one
        // site, the site leaving it taken from the row's other word
        const bool left = (hf == 0) != ((k & 1) != 0);
        uint32_t side;
        if constexpr (kWq == 1) {
          side = left ? __funnelshift_l(ctr, ctr, 1) : __funnelshift_r(ctr, ctr, 1);
        } else {
          const uint32_t other = ob[(y0 + k + 1) * kWq + (c ^ 1) - c];
          side = left ? __funnelshift_l(other, ctr, 1) : __funnelshift_r(ctr, other, 1);
        }
        count_masks(s, ctr, side, o[k], o[k + 2], av[k], ac[k]);
        un[k] = valid ? 0xFFFFFFFFu - ac[k] : 0u;  // = ~ac, on the FMA pipe
        site[k] = (uint32_t)(ti * GW + g) * (uint32_t)wpp + (uint32_t)((y0 + k) * kWq + c);  // word number
      }
      const uint32_t chain = ((uint32_t)ti * blockDim.x + (uint32_t)tid) * 8u;
      accept_native(av, un, ac, site, chain, c1, (uint32_t)P.step, P.tag, keys, s_dig, valid ? kKB : 0, P.T4, P.T8);
      if (valid) {
#pragma unroll
        for (int k = 0; k < kKB; ++k) {
          const int y = y0 + k;
          const uint32_t nw = sb[y * kWq] ^ ac[k];
          sb[y * kWq] = nw;
          if (y == 0) sb[kL * kWq] = nw;       // copy below row L-1
          if (y == kL - 1) sb[-kWq] = nw;      // copy above row 0
        }
      }
    };
    const bool full_word = full_rows(Wq, seg);  // block-uniform (L = 64 or 128)
    const int sweeps = P.sweeps;
    for (int sw = 0; sw < sweeps; ++sw) {
#pragma unroll 1
      for (int hf = 0; hf < 2; ++hf) {
        uint32_t* self = pl + hf * GW * P.gs;
        const uint32_t* oth = pl + (1 - hf) * GW * P.gs;
        const uint32_t c1 = (uint32_t)((sw * 2 + hf) << 4);
        if (full_word && Wq == 1) half_full(std::integral_constant<int, 1>(), self, oth, hf, c1);
        else if (full_word) half_full(std::integral_constant<int, 2>(), self, oth, hf, c1);
        else half_sweep(self, oth, hf, c1);
        __syncthreads();
      }
    }

    }

    bits_count(P, pl, ti, s_anti, s_plus);
    bits_move(P, pl, ti, false);
    __syncthreads();
    {
      const int r0 = ti * P.G, gc = bits_present(P, ti), N = P.N;
      for (int j = tid; j < gc; j += blockDim.x) {
        P.E[r0 + j] = -2 * N + 2 * s_anti[j];
        P.M[r0 + j] = 2 * s_plus[j] - N;
      }
      if (tid < kMsb)
        for (int j = tid; j < gc; j += kMsb) stats.add(tid, -2 * N + 2 * s_anti[j], 2 * s_plus[j] - N);
    }
  }
  if (tid < kMsb && cur >= 0) stats.flush(b->pops + cur, tid);
}

cudaError_t ssc_bits_setup(int smem, SweepLaunch* out) {
  return persistent_launch((const void*)ssc_sweep_bits_kernel, kSweepThreads, smem, out);
}

cudaError_t launch_ssc_bits_sweep(BatchDev* b, int energy_only, unsigned long long seed, const SweepLaunch& sl,
                                  cudaStream_t s) {
  ssc_sweep_bits_kernel<<<sl.grid, sl.block, sl.smem, s>>>(b, energy_only, PhiloxKeysWide(seed));
  return cudaGetLastError();
}

}  // namespace pa
