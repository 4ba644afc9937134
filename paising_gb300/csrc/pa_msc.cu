// pa_msc.cu -- multi-spin coding: 32 replicas bit-packed per uint32 word.
//
// Replaces, from the reference PAisingMSC.cu (MSbits = 32):
//   ReplicaInit  (PAisingMSC.cu:169-188)  -> msc_init_kernel
//   checkKerALL  (PAisingMSC.cu:191-266)  -> msc_sweep_kernel (group resident in
//   energyKer    (PAisingMSC.cu:268-317)     shared memory for all sweeps; per
//                                            replica energy and magnetisation by
//                                            bitsliced counters in the epilogue)
//   resampleKer  (PAisingMSC.cu:397-435)  -> msc_resample_kernel (gather: each new
//                                            word assembles its 32 source bits,
//                                            no atomics, no memset)
//
// Layout in HBM: group g occupies N words at spins + g*N (sublattice A words,
// then B); bit k of a word is replica k of the group, 1 == spin +1.
#include <algorithm>
#include <climits>
#include <type_traits>

#include "pa_kernels.h"
#include "pa_msc_core.cuh"

namespace pa {

using namespace msc;

// ------------------------------------------------------------------ init
__global__ void msc_init_kernel(PopDev* pops) {
  PopDev* st = pops + blockIdx.y;
  const int N = st->N, h = N >> 1, R = st->R_cur, rg = (R + kMsb - 1) / kMsb;
  const unsigned long long seed = st->seed, iseq = st->iseq;
  uint32_t* wd = (uint32_t*)st->spins[st->parity];
  uint8_t* act = st->active[st->parity];
  if (st->init_src) {  // caller-supplied population (replica 32g+k at group g, bit k)
    const uint4* src = (const uint4*)st->init_src;
    uint4* dst = (uint4*)wd;
    const long long nv = (long long)rg * N / 4;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nv; v += (long long)gridDim.x * blockDim.x)
      dst[v] = src[v];
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < (long long)rg * kMsb;
         i += (long long)gridDim.x * blockDim.x)
      act[i] = i < R;
    return;
  }
  // ReplicaInit (PAisingMSC.cu:169-188): reference thread t of block B draws
  // words 2k (gA) and 2k+1 (gB) of subsequence iseq + t + 128 B for idx = t + 128 k
  const long long total = (long long)rg * h;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int g = (int)(e / h), idx = (int)(e - (long long)g * h);
    const int t = idx & (kRefThreads - 1), k = idx >> 7;
    const unsigned long long sub = iseq + (unsigned long long)t + (unsigned long long)kRefThreads * g;
    wd[(size_t)g * N + idx] = ref_word(seed, sub, 2ull * k);
    wd[(size_t)g * N + h + idx] = ref_word(seed, sub, 2ull * k + 1);
    if (idx < kMsb) act[g * kMsb + idx] = (g * kMsb + idx) < R;
  }
}

// ----------------------------------------------------------------- sweep
// Persistent: every CTA takes tiles of G groups of 32 replicas of any
// population from the batch's work queue and anneals one tile at a time,
// resident in shared memory as all G sublattices A, then all G sublattices B
// (so the tile is one stack of G*L sublattice rows of Wr words; a row's
// vertical neighbours wrap inside its own group).  Thread (rsub, tx) owns
// word column tx of stacked rows rsub, rsub+rpp, ...; with one group per
// tile (G = 1) in the native stream it owns the consecutive rows
// rsub*npass .. rsub*npass + npass - 1 instead, and each sublattice carries
// periodic copies of rows -1 and L (msc_move_tile), so that a batch of four
// rows shares its six rows of the other sublattice and nothing wraps.
//
// MODE kRefCoords: decisions of checkKerALL exactly -- one draw per word-site
//   (ctr = sw*2K + hf*K + k of subsequence iseq + t + 128 g) expanded to 32
//   numbers by the LCG and compared with T4 = ceil(2^32 e^-4b), T8.
// MODE kNative: U_i < T/2^32 for the 32 replica bits is decided digit by
//   digit, most significant first, each digit a fresh Philox4x32-10 bit
//   (accept_native); each replica's acceptance probability is exactly
//   T/2^32, as in the reference.  The stream is keyed by stream_seed (one
//   per batch; populations differ in counter word 3).
// Tile gi0 (gc groups present) <-> HBM.  G > 1 (implies h % 4 == 0): group
// gi0+g's sublattice X goes to lat + X*G*h + g*h.  G = 1: sublattice X is a
// block of L + 2 rows at lat + X*sb -- row -1 (a copy of row L-1), rows
// 0..L-1, row L (a copy of row 0) -- so that the native sweep reads its
// vertical neighbours without wrapping; the sweep keeps the copies current.
// Out of line: keeps the sweep loop's registers free.
__device__ __noinline__ void msc_move_tile(const UnitParams& P, uint32_t* lat, int gi0, int gc, bool to_smem) {
  const int N = P.N, h = P.h, G = P.G;
  uint4* lat4 = (uint4*)lat;
  uint4* g4 = (uint4*)(P.words + (size_t)gi0 * N);
  if (G == 1) {
    const int Wr = P.Wr, L = P.L;
    uint32_t* gw = P.words + (size_t)gi0 * N;
    if ((Wr & 3) == 0) {  // rows start on 16-byte boundaries in both places
      const int h4 = h >> 2;
      for (int v = threadIdx.x; v < 2 * h4; v += blockDim.x) {
        const int X = v >= h4 ? 1 : 0, i = v - X * h4;
        uint4* s = (uint4*)(lat + X * P.sb + Wr) + i;
        uint4* d = (uint4*)(gw + X * h) + i;
        if (to_smem) *s = *d;
        else *d = *s;
      }
    } else {
      for (int v = threadIdx.x; v < N; v += blockDim.x) {
        const int X = v >= h ? 1 : 0, i = v - X * h;
        uint32_t* s = lat + X * P.sb + Wr + i;
        if (to_smem) *s = gw[v];
        else gw[v] = *s;
      }
    }
    if (to_smem)  // periodic copies: row -1 = row L-1, row L = row 0
      for (int v = threadIdx.x; v < 4 * Wr; v += blockDim.x) {
        const int X = v >= 2 * Wr ? 1 : 0, r = v - X * 2 * Wr, top = r < Wr ? 1 : 0, i = top ? r : r - Wr;
        lat[X * P.sb + (top ? 0 : (L + 1) * Wr) + i] = gw[X * h + (top ? (L - 1) * Wr : 0) + i];
      }
    return;
  }
  const int h4 = h >> 2, n4 = N >> 2;
  for (int v = threadIdx.x; v < 2 * gc * h4; v += blockDim.x) {
    const int X = v >= gc * h4 ? 1 : 0, r = v - X * gc * h4;
    const int g = (int)__umulhi((uint32_t)r, P.invH4), i = r - g * h4;
    uint4* s = lat4 + X * G * h4 + g * h4 + i;
    uint4* d = g4 + (size_t)g * n4 + X * h4 + i;
    if (to_smem) *s = *d;
    else *d = *s;
  }
}

// Energy and magnetisation per replica bit of the tile: the left and up
// bond of every A and B site (PAisingMSC.cu:272-294), counted per bit in
// bitsliced counters (BitCounters) and added into cntE / cntM [group of the
// tile][bit].  Each warp works inside one group (kSweepThreads/32/G warps per
// group, at most h / (32 wpg) <= 32 words per lane), so its counts never mix
// groups.
__device__ __noinline__ void msc_count(const UnitParams& P, const uint32_t* lat, int gc, int* cntE, int* cntM) {
  const int tid = threadIdx.x, lane = tid & 31;
  const int L = P.L, Wr = P.Wr, h = P.h, G = P.G, wpg = (kSweepThreads / 32) / G;
  const int w = tid >> 5, g = w / wpg, ws = w - g * wpg;
  if (g >= gc) return;  // warp-uniform
  BitCounters bc;
  bc.reset();
  const uint32_t* A = G == 1 ? lat + Wr : lat + g * h;
  const uint32_t* B = G == 1 ? lat + P.sb + Wr : lat + G * h + g * h;
  for (int j0 = ws * 32; j0 < h; j0 += wpg * 32) {
    const int j = j0 + lane;
    uint32_t s0 = 0, s1 = 0, s2 = 0, sA = 0, sB = 0;
    if (j < h) {
      const int y = (int)__umulhi((uint32_t)j, P.invWr), x = j - y * Wr;
      const int iL = y * Wr + (x == 0 ? Wr - 1 : x - 1), iU = (y + 1 == L ? 0 : y + 1) * Wr + x;
      sA = A[j];
      sB = B[j];
      uint32_t Ai2, Bi2;
      if (y & 1) { Ai2 = sB; Bi2 = A[iL]; }
      else { Ai2 = B[iL]; Bi2 = sA; }
      adder4(sA ^ Ai2, sA ^ B[iU], sB ^ Bi2, sB ^ A[iU], s0, s1, s2);
    }
    bc.add(s0, s1, s2, sA, sB);
  }
  int cE, cM;  // lane k: bit k
  bc.totals(lane, cE, cM);
  atomicAdd(&cntE[g * kMsb + lane], cE);
  atomicAdd(&cntM[g * kMsb + lane], cM);
}

static_assert(kMaxTile * kMsb == kSweepThreads, "one thread per (group of the tile, bit) in the epilogue");
// FL != 0 (native stream only): a kernel for populations of lattice size FL
// with one group per work unit, holding that size's compile-time sweep alone.
// Built for L = 96 only: the general kernel (FL = 0) carries the compile-time
// forms of L = 64 and 128, measured as fast there as kernels of their own,
// while adding L = 96's form to it cost L = 64 2.4% (register allocation).
// FL = kWith96 is the general kernel with L = 96's form as well, for batches
// that mix L = 96 with other sizes (64 uneven populations: 2% faster than the
// general kernel; L = 96 beside L = 64: 7%).
template <int MODE, int FL>
__global__ void __launch_bounds__(kSweepThreads, 4)
    msc_sweep_kernel(BatchDev* b, int energy_only, unsigned long long stream_seed) {
  const PhiloxKeys keys(stream_seed);
  extern __shared__ __align__(16) uint32_t lat[];  // G*N words: G sublattices A, then G sublattices B
  __shared__ int s_unit, s_pop;
  __shared__ int s_cntE[kMaxTile * kMsb], s_cntM[kMaxTile * kMsb];  // [group of the tile][bit]
  __shared__ uint2 s_dig[kMsb];  // per digit j: digit_table(T4, T8, j)
  __shared__ UnitParams P;
  __shared__ BitStats stats;

  const int tid = threadIdx.x, lane = tid & 31;
  const int total = b->unit_prefix[b->npop];
  int cur = -1;
  int tx = 0, rsub = 0, txl = 0, txr = 0;
  bool worker = false;
  if (tid < kMsb) stats.reset(tid);

  for (;;) {
    __syncthreads();
    if (tid == 0) {
      const int u = (int)atomicAdd(&b->work_next, 1u);
      int loc = 0;
      const int p = u < total ? queue_pop(b, u, &loc) : -1;
      s_pop = p;
      s_unit = loc;
      if (p >= 0 && p != cur) {  // parameters of a new population
        const PopDev* st = b->pops + p;
        P.L = st->L; P.N = st->N; P.h = st->N >> 1; P.Wr = st->Wr; P.rpp = st->rpp; P.npass = st->npass;
        P.kconst = st->kconst;
        P.step = (int)native_step_word(st);
        P.sweeps = energy_only ? 0 : st->sweeps;
        P.nbatch = (st->npass + kKB - 1) / kKB;
        P.G = st->gpt > 0 ? st->gpt : 1;
        P.rg = (st->R_cur + kMsb - 1) / kMsb;
        P.sb = msc_halo_block(st->L, st->Wr);
        P.invL = st->invL;
        P.invWr = st->invWr;
        const unsigned long long h4 = (unsigned long long)(st->N >> 3);
        P.invH4 = (uint32_t)((0x100000000ull + h4 - 1) / h4);
        P.tag = kTagMscSweep | (uint32_t)st->pop_id;
        P.T4 = st->thr[(size_t)st->step * kThrPerStep + 10];
        P.T8 = st->thr[(size_t)st->step * kThrPerStep + 11];
        P.seed = st->seed;
        const int rg_prev = (st->R_prev + kMsb - 1) / kMsb;
        P.iseq = st->iseq + (st->step > 0 ? (unsigned long long)rg_prev * kMsb : 0ull);
        P.words = (uint32_t*)st->spins[st->parity];
        P.act = st->active[st->parity];
        P.E = st->E;
        P.M = st->M;
      }
    }
    s_cntE[tid] = 0;  // kMaxTile * kMsb == kSweepThreads
    s_cntM[tid] = 0;
    __syncthreads();
    const int p = s_pop, ti = s_unit;  // population, tile
    if (p < 0) break;
    if (p != cur) {  // block-uniform
      if (tid < kMsb && cur >= 0) stats.flush(b->pops + cur, tid);
      cur = p;
      const int Wr = P.Wr;
      worker = tid < Wr * P.rpp;
      tx = worker ? tid % Wr : 0;
      rsub = worker ? tid / Wr : 0;
      txl = (tx == 0 ? Wr - 1 : tx - 1);
      txr = (tx + 1 == Wr ? 0 : tx + 1);
      if (tid < kMsb) {
        s_dig[tid] = digit_table(P.T4, P.T8, tid);
      }
    }
    const int N = P.N, h = P.h, G = P.G, gi0 = ti * G;
    const int gc = min(G, P.rg - gi0);  // groups present in this tile
    msc_move_tile(P, lat, gi0, gc, true);
    __syncthreads();

    // stacked row v of the tile -> group g, row y in the group, smem offsets
    // of the row and its vertical neighbours (periodic inside the group)
    struct RowPos {
      int g, y, row, rowu, rowd;
    };
    auto row_pos = [&](int v) {
      RowPos q;
      const int L = P.L, Wr = P.Wr;
      q.g = (int)__umulhi((uint32_t)v, P.invL);
      q.y = v - q.g * L;
      q.row = v * Wr;
      q.rowu = (q.y == 0 ? v + L - 1 : v - 1) * Wr;
      q.rowd = (q.y + 1 == L ? v + 1 - L : v + 1) * Wr;
      return q;
    };
    const int vrows = gc * P.L;  // stacked rows present
    const int sweeps = P.sweeps;
    for (int sw = 0; sw < sweeps; ++sw) {
#pragma unroll 1
      for (int hf = 0; hf < 2; ++hf) {
        // row 0 of the swept and of the other sublattice
        uint32_t* self = G == 1 ? lat + (hf ? P.sb : 0) + P.Wr : lat + (hf ? G * h : 0);
        const uint32_t* oth = G == 1 ? lat + (hf ? 0 : P.sb) + P.Wr : lat + (hf ? 0 : G * h);
        const int Wr = P.Wr, rpp = P.rpp, npass = P.npass;
        if (MODE == kRefCoords) {
#pragma unroll 1
          for (int pass = 0; pass < npass; ++pass) {
            const int v = rsub + pass * rpp;
            const bool valid = worker && v < vrows;
            const RowPos q = row_pos(valid ? v : 0);
            const int sidx = q.row + tx;       // word in the tile's sublattice array
            const int idx = q.y * Wr + tx;     // word in the group's sublattice
            const int gi = gi0 + q.g;
            // horizontal neighbour not at the same idx (PAisingMSC.cu:203, 238)
            const bool left = (hf == 0) == ((q.y & 1) == 0);
            const uint32_t s = self[sidx];
            const uint32_t n1 = oth[q.row + (left ? txl : txr)], n2 = oth[sidx], n3 = oth[q.rowu + tx],
                           n4 = oth[q.rowd + tx];
            uint32_t s0, s1, s2;
            adder4(s ^ n1, s ^ n2, s ^ n3, s ^ n4, s0, s1, s2);
            const int t = idx & (kRefThreads - 1), k = idx >> 7;
            const int K = P.kconst ? P.kconst : (t < h ? (h - t + kRefThreads - 1) / kRefThreads : 0);
            const unsigned long long sub = P.iseq + (unsigned long long)t + (unsigned long long)kRefThreads * gi;
            uint32_t ran = ref_word(P.seed, sub, (unsigned long long)sw * 2 * K + (unsigned long long)hf * K + k);
            const uint32_t T4 = P.T4, T8 = P.T8;
            uint32_t c4 = 0, c8 = 0;
#pragma unroll 8
            for (int i = 0; i < kMsb; ++i) {
              c4 |= (ran < T4 ? 1u : 0u) << i;
              c8 |= (ran < T8 ? 1u : 0u) << i;
              ran = kLcgA * ran + kLcgC;
            }
            const uint32_t hi = s1 | s2;
            const uint32_t acc = hi | (~hi & ((s0 & c4) | (~s0 & c8)));
            if (valid) self[sidx] = s ^ acc;
          }
        } else {
          const uint32_t c1 = (uint32_t)((sw * 2 + hf) << 4);
          const uint32_t base = (uint32_t)gi0 * (uint32_t)h;  // site number of the tile's first word
          // L = 64, 96 and 128 with every size fixed at compile time: kW = L/2
          // words per row, kR = kSweepThreads/kW thread rows of kRows =
          // ceil(kL/kR) consecutive rows each (64: a warp per row, 8 rows per
          // thread; 96: 5 x 20 rows, the last batch of the fifth thread row
          // past the lattice; 128: two warps per row, 32 rows per thread);
          // every offset an immediate.  Same batches as the general form.
          auto native_fixed = [&](auto l_c) {
            constexpr int kL = decltype(l_c)::value, kW = kL / 2, kR = kSweepThreads / kW;
            constexpr int kRows = (kL + kR - 1) / kR;
            static_assert(kRows % kKB == 0 && (kR * kRows - kL) % kKB == 0, "whole batches, each in or past the lattice");
            const int vb0 = rsub * kRows;
            const uint32_t* txs = oth + (hf == 0 ? txl : txr);  // side neighbour on even rows
            const uint32_t* txo = oth + (hf == 0 ? txr : txl);  // and on odd rows
#pragma unroll 1
            for (int p0 = 0; p0 < kRows; p0 += kKB) {
              // a batch past the lattice (or of a thread without a column)
              // reads rows 0..3 and decides nothing, but takes part in the
              // warp's acceptance
              constexpr bool kAll = kR * kW == kSweepThreads && kR * kRows == kL;  // every batch of every thread
              const bool bvalid = kAll || (worker && vb0 + p0 < kL);
              const int vb = bvalid ? vb0 + p0 : 0;
              const uint32_t* po = oth + (vb - 1) * kW + tx;  // rows vb-1 .. vb+4 (rows -1 and kL: copies)
              uint32_t* ps = self + vb * kW + tx;
              uint32_t av[kKB], un[kKB], ac[kKB], site[kKB];
#pragma unroll
              for (int k = 0; k < kKB; ++k) {
                const uint32_t s = ps[k * kW];
                const uint32_t side = ((k & 1) ? txo : txs)[(vb + k) * kW];
                count_masks(s, side, po[(k + 1) * kW], po[k * kW], po[(k + 2) * kW], av[k], ac[k]);
                un[k] = bvalid ? 0xFFFFFFFFu - ac[k] : 0u;  // = ~ac, on the FMA pipe
                site[k] = base + (uint32_t)((vb + k) * kW + tx);
              }
              const uint32_t chain =
                  ((uint32_t)ti * blockDim.x + (uint32_t)tid) * (uint32_t)(kRows / kKB) + (uint32_t)(p0 / kKB);
              accept_native(av, un, ac, site, chain, c1, (uint32_t)P.step, P.tag, keys, s_dig, kKB, P.T4, P.T8);
              if (bvalid) {
#pragma unroll
                for (int k = 0; k < kKB; ++k) {
                  const uint32_t nw = ps[k * kW] ^ ac[k];
                  ps[k * kW] = nw;
                  if (vb + k == 0) self[kL * kW + tx] = nw;         // copy below row kL-1
                  if (vb + k == kL - 1) self[-kW + tx] = nw;        // copy above row 0
                }
              }
            }
          };
          if constexpr (FL > kWith96) {
            if (G == 1 && P.L == FL) {  // block-uniform; anything else is a host error, recorded below
              native_fixed(std::integral_constant<int, FL>());
            } else if (tid == 0 && sw == 0 && hf == 0) {
              b->pops[p].error = kErrSweepForm;
            }
          } else if (G == 1 && P.L == 64) {
            native_fixed(std::integral_constant<int, 64>());
          } else if (G == 1 && P.L == 128) {
            native_fixed(std::integral_constant<int, 128>());
          } else if (FL == kWith96 && G == 1 && P.L == 96) {
            native_fixed(std::integral_constant<int, 96>());
          } else if (G == 1) {
            // one group, any other L: thread rsub owns the
            // consecutive rows rsub*npass .. rsub*npass + npass - 1 of column
            // tx, so a batch of kKB rows shares the other sublattice's rows
            // around them, and the periodic copies of rows -1 and L spare the
            // vertical wrap
            const int L = P.L;
#pragma unroll 1
            for (int p0 = 0; p0 < npass; p0 += kKB) {
              const int vb = rsub * npass + p0;  // first row of the batch
              uint32_t o[kKB + 2];  // other sublattice, rows vb-1 .. vb+kKB (clamped to the copy of row 0)
#pragma unroll
              for (int j = 0; j < kKB + 2; ++j) o[j] = oth[min(vb - 1 + j, L) * Wr + tx];
              // horizontal neighbour not at the same index: left for A on even
              // rows and B on odd rows (PAisingMSC.cu:203, 238); alternates by row
              const bool left0 = (hf == 0) == ((vb & 1) == 0);
              uint32_t av[kKB], un[kKB], ac[kKB], site[kKB];
              uint32_t vm = 0;  // slots holding a site
#pragma unroll
              for (int k = 0; k < kKB; ++k) {
                const int y = vb + k;
                const bool valid = worker && p0 + k < npass && y < L;
                const int row = min(y, L) * Wr;
                const uint32_t s = self[row + tx];
                const uint32_t side = oth[row + ((left0 != ((k & 1) != 0)) ? txl : txr)];
                count_masks(s, side, o[k + 1], o[k], o[k + 2], av[k], ac[k]);
                un[k] = valid ? 0xFFFFFFFFu - ac[k] : 0u;  // = ~ac, on the FMA pipe
                vm |= valid ? 1u << k : 0u;
                site[k] = base + (uint32_t)(row + tx);  // = group * h + word in the group
              }
              const uint32_t chain = ((uint32_t)ti * blockDim.x + (uint32_t)tid) * (uint32_t)P.nbatch + (uint32_t)(p0 / kKB);
              accept_native(av, un, ac, site, chain, c1, (uint32_t)P.step, P.tag, keys, s_dig, npass - p0, P.T4, P.T8);
#pragma unroll
              for (int k = 0; k < kKB; ++k)
                if (vm >> k & 1u) {
                  const int y = vb + k;
                  const uint32_t nw = self[y * Wr + tx] ^ ac[k];
                  self[y * Wr + tx] = nw;
                  if (y == 0) self[L * Wr + tx] = nw;         // copy below row L-1
                  if (y == L - 1) self[-Wr + tx] = nw;        // copy above row 0
                }
            }
          } else {
            // stacked tiles: thread (rsub, tx) takes stacked rows rsub + pass*rpp
#pragma unroll 1
            for (int p0 = 0; p0 < npass; p0 += kKB) {
              uint32_t av[kKB], un[kKB], ac[kKB], site[kKB];
              uint32_t vm = 0;  // slots holding a site
#pragma unroll
              for (int k = 0; k < kKB; ++k) {
                const int pass = p0 + k;
                const int v = rsub + pass * rpp;
                const bool valid = worker && pass < npass && v < vrows;
                const int vc = valid ? v : 0;
                const RowPos q = row_pos(vc);
                const int sidx = q.row + tx;
                // row parity: stacked groups have even L, so v and y agree
                const bool left = (hf == 0) == ((vc & 1) == 0);
                const uint32_t s = self[sidx];
                const uint32_t n1 = oth[q.row + (left ? txl : txr)], n2 = oth[sidx], n3 = oth[q.rowu + tx],
                               n4 = oth[q.rowd + tx];
                count_masks(s, n1, n2, n3, n4, av[k], ac[k]);
                un[k] = valid ? 0xFFFFFFFFu - ac[k] : 0u;  // = ~ac, on the FMA pipe
                vm |= valid ? 1u << k : 0u;
                site[k] = base + (uint32_t)sidx;  // = group * h + word in the group
              }
              const uint32_t chain = ((uint32_t)ti * blockDim.x + (uint32_t)tid) * (uint32_t)P.nbatch + (uint32_t)(p0 / kKB);
              accept_native(av, un, ac, site, chain, c1, (uint32_t)P.step, P.tag, keys, s_dig, npass - p0, P.T4, P.T8);
#pragma unroll
              for (int k = 0; k < kKB; ++k)
                if (vm >> k & 1u) self[site[k] - base] ^= ac[k];
            }
          }
        }
        __syncthreads();
      }
    }

    msc_count(P, lat, gc, s_cntE, s_cntM);
    msc_move_tile(P, lat, gi0, gc, false);
    __syncthreads();
    if (tid < gc * kMsb) {
      const int gi = gi0 + (tid >> 5);
      const int E = 2 * s_cntE[tid] - 2 * N, Mg = 2 * s_cntM[tid] - N;
      P.E[gi * kMsb + lane] = E;
      P.M[gi * kMsb + lane] = Mg;
    }
    if (tid < kMsb) {  // lane k of warp 0 owns the statistics of bit k
      for (int g = 0; g < gc; ++g) {
        const int gi = gi0 + g, E = 2 * s_cntE[g * kMsb + tid] - 2 * N, Mg = 2 * s_cntM[g * kMsb + tid] - N;
        if (P.act[gi * kMsb + tid]) stats.add(tid, E, Mg);
      }
    }
  }
  if (tid < kMsb && cur >= 0) stats.flush(b->pops + cur, tid);
}

// -------------------------------------------------------------- resample
// Reference stream: resampleKer places offspring number s (in the scan order
// of (old group, bit)) at new group s % rg_new, bit s / rg_new
// (PAisingMSC.cu:413-414), which the reference-stream parity needs.  Here every new word gathers its 32 bits:
// bit k of new group j comes from old replica src[k*rg_new + j].
//
// Work unit of one warp: 32 consecutive new groups (lane g builds group
// j0 + g) x a strip of 32 sites.  Lane g resolves the sources of its 32 bits
// into row pointers and rotations held in registers, four bits at a time,
// and gathers its 32 output words with loads at immediate offsets.  The 32
// lanes' sources are 32 consecutive new replicas, i.e. neighbouring old
// replicas in one or two old groups, so a load instruction touches one or two
// old words: the gather costs about one warp load per output word, and no L2
// traffic beyond the old rows themselves.  Units of all populations of the
// batch come from one queue (msc_resample_plan_kernel) and are taken by
// persistent warps, so uneven populations finish together.
constexpr int kResampleThreads = 256;
constexpr int kSub = 8;  // sites gathered per pass over the 32 source bits

// Sites per warp unit: 32, or 8 when a population would otherwise have too
// few units to occupy the GPU (small lattices).
__device__ __forceinline__ int res_strip(int N, int rgn) {
  const int tiles = (rgn + 31) / 32;
  return (long long)tiles * (N / 32) >= 8192 ? 32 : kSub;
}

// Native stream gather (msc_resample_native_kernel): units of kNatGroups new
// groups x kNatSites sites.
constexpr int kNatGroups = 16;      // new groups per unit of the native gather
constexpr int kNatBatch = 2;        // of which staged and gathered together
constexpr int kNatThreads = 256;
constexpr int kNatBlocksPerSM = 4;

constexpr int kNatSites = 64;       // sites per unit (two per lane)

__device__ __forceinline__ int nat_units(int N, int rgn) {
  return ((rgn + kNatGroups - 1) / kNatGroups) * ((N + kNatSites - 1) / kNatSites);
}

__global__ void __launch_bounds__(1024) msc_resample_plan_kernel(BatchDev* b, int native) {
  __shared__ uint32_t s_u[33];
  const int p = threadIdx.x, np = b->npop;
  uint32_t units = 0, groups = 0;
  if (p < np) {
    const PopDev* st = b->pops + p;
    if (st->coding == kMSC && pop_stepping(st)) {
      const int rgn = (st->R_cur + kMsb - 1) / kMsb, S = res_strip(st->N, rgn);
      units = native ? (uint32_t)nat_units(st->N, rgn)
                                      : (uint32_t)(((rgn + 31) / 32) * ((st->N + S - 1) / S));
      groups = (uint32_t)rgn;
    }
  }
  uint32_t total, gtotal;
  const uint32_t ex = block_exscan(units, s_u, &total);
  __syncthreads();  // s_u is reused
  const uint32_t gex = block_exscan(groups, s_u, &gtotal);
  if (p < np) {
    b->res_prefix[p] = (int)ex;
    b->grp_prefix[p] = (int)gex;
  }
  if (p == 0) {
    b->res_prefix[np] = (int)total;
    b->grp_prefix[np] = (int)gtotal;
    b->res_next = 0;
  }
}

template <bool kFull>
__device__ __forceinline__ void gather_sub(const uint32_t* const (&p)[4], const uint32_t (&rot)[4],
                                           const uint32_t (&msk)[4], int nv, uint32_t (&w)[kSub]) {
#pragma unroll
  for (int t = 0; t < kSub; ++t) {
    const int tc = kFull ? t : min(t, nv - 1);  // partial: repeat the last site (not stored)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const uint32_t v = __ldg(p[q] + tc);
      w[t] |= __funnelshift_l(v, v, rot[q]) & msk[q];  // source bit rotated into bit k
    }
  }
}

constexpr int kResampleBlocksPerSM = 3;  // 80 registers, no spills

__global__ void __launch_bounds__(kResampleThreads, kResampleBlocksPerSM) msc_resample_kernel(BatchDev* b) {
  const int lane = threadIdx.x & 31;
  const int total = b->res_prefix[b->npop];
  for (;;) {
    int u = 0;
    if (lane == 0) u = (int)atomicAdd(&b->res_next, 1u);
    u = __shfl_sync(kFull, u, 0);
    if (u >= total) break;
    int lo = 0, hi = b->npop;  // population of unit u
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (b->res_prefix[mid] <= u) lo = mid;
      else hi = mid;
    }
    const PopDev* st = b->pops + lo;
    const int N = st->N, Rn = st->R_cur, rgn = (Rn + kMsb - 1) / kMsb, S = res_strip(N, rgn);
    const int nstrip = (N + S - 1) / S;
    const int loc = u - b->res_prefix[lo], tile = loc / nstrip, strip = loc - tile * nstrip;
    const int j = tile * 32 + lane, t0 = strip * S, nt = min(S, N - t0);
    const bool jv = j < rgn;
    const uint32_t* old = (const uint32_t*)st->spins[st->parity ^ 1];
    const uint32_t* src = st->src;
    if (strip == 0 && jv) {
      uint8_t* act = st->active[st->parity];
#pragma unroll 4
      for (int k = 0; k < kMsb; ++k) act[j * kMsb + k] = (k * rgn + j) < Rn ? 1 : 0;
    }
    uint32_t* dst = (uint32_t*)st->spins[st->parity] + (size_t)j * N + t0;
#pragma unroll 1
    for (int tc = 0; tc < nt; tc += kSub) {
      const int nv = min(kSub, nt - tc);  // a multiple of 4: N and t0 are
      uint32_t w[kSub];
#pragma unroll
      for (int t = 0; t < kSub; ++t) w[t] = 0u;
#pragma unroll 1
      for (int k0 = 0; k0 < kMsb; k0 += 4) {
        const uint32_t* p[4];
        uint32_t rot[4], msk[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int k = k0 + q, s = k * rgn + j;
          const bool v = jv && s < Rn;
          const uint32_t lin = v ? src[s] : 0u;  // an invalid bit reads old word 0 and is masked off
          p[q] = old + (size_t)(lin >> 5) * N + t0 + tc;
          rot[q] = ((uint32_t)k - (lin & 31u)) & 31u;
          msk[q] = v ? 1u << k : 0u;
        }
        if (nv == kSub) gather_sub<true>(p, rot, msk, nv, w);
        else gather_sub<false>(p, rot, msk, nv, w);
      }
      if (jv) {
        uint4* d4 = reinterpret_cast<uint4*>(dst + tc);
        d4[0] = make_uint4(w[0], w[1], w[2], w[3]);
        if (nv > 4) d4[1] = make_uint4(w[4], w[5], w[6], w[7]);
      }
    }
  }
}

// --------------------------------------------- resample, native stream
// With the engine's own stream the placement of offspring is free (replicas
// are exchangeable), so offspring s goes to slot s: group s / 32, bit s % 32.
// The sources of a new group's 32 bits are then 32 consecutive entries of the
// monotone gather map, i.e. a window of old replicas that are mostly
// consecutive themselves: with offsets o_b = src[32j + b] - 32 (first - 1),
// first = src[32j] / 32, bit b of the new word is bit o_b of the bit string
// W = old words first-1, first, first+1, first+2 at that site (W's word 0 is
// never selected: o_b >= 32).  Bits sharing the shift d = o_b - b form one
// mask M_d, and the new word is OR_d ((W >> d) & M_d), one funnel shift and
// one logic operation per distinct shift instead of per bit.  Copy numbers
// of 1 keep the shift; a duplicate lowers it by one, a replica without
// offspring raises it, so a word has a handful of distinct shifts.
//
// Copies of one parent are the exception: a run of k new bits with the same
// source has k distinct shifts, so a parent with many copies (a large dbeta
// against the energy spread) would turn a word into 32 single-bit pairs.
// A run of four or more is one broadcast pair instead: the run's mask M and
// the source's position p in the window, new |= M & -(bit p of W).
//
// msc_pairs_kernel (one warp per new group of every population, lane b for
// bit b) lists a group's distinct shifts of the other bits as (M_d, d mod 32)
// pairs ordered by the window word d / 32 they start in (counts n0, n1, n2),
// then its runs of four or more bits of one source as (M, 31 - p mod 32)
// pairs ordered by the window word p / 32 holding the source (counts k1, k2,
// k3): the lanes sharing a shift or a source find each other with one match
// each, and the lowest of them writes the pair.  A group whose sources span more than the
// four-word window (more than 64 replicas without offspring among ~96
// consecutive ones), or whose counts do not fit the 5-bit fields of its count
// word, is flagged and gathered bit by bit.
__global__ void __launch_bounds__(256) msc_pairs_kernel(BatchDev* b) {
  const int lane = threadIdx.x & 31, np = b->npop, total = b->grp_prefix[np];
  const uint32_t lt = (1u << lane) - 1u;
  for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < total; i += (gridDim.x * blockDim.x) >> 5) {
    int lo = 0, hi = np;  // population of new group i (warp-uniform)
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (b->grp_prefix[mid] <= i) lo = mid;
      else hi = mid;
    }
    PopDev* st = b->pops + lo;
    const int j = i - b->grp_prefix[lo], nb = min(kMsb, st->R_cur - j * kMsb);
    const uint32_t* src = st->src + (size_t)j * kMsb;
    const bool v = lane < nb;
    // source of bit b relative to the window, o = src[b] - 32 (first - 1) >= 32
    // (src nondecreasing, src[0] >= 32 first), and its shift d = o - b >= 1
    const uint32_t base = ((src[0] >> 5) - 1u) * 32u;  // may wrap; only differences matter
    const uint32_t s = v ? src[lane] : 0xFFFFFFFFu;    // the invalid bits share 0xFFFFFFFF
    const uint32_t o = s - base, d = o - (uint32_t)lane;
    bool fallback = __any_sync(kFull, v && d >= 96u);  // then o < 128 for every bit
    // bits with this bit's source; a run of k >= 4 of them is one broadcast
    // pair (as shifts its first and last bits join their neighbours' pairs,
    // the k - 2 between take a pair each)
    const uint32_t ms = __match_any_sync(kFull, s);
    const bool run = v && __popc(ms) >= 4;
    const uint32_t m = __match_any_sync(kFull, v && !run ? d : 0xFFFFFFFFu);  // bits outside runs with this shift
    const bool lead_d = v && !run && (m & lt) == 0u, lead_r = run && (ms & lt) == 0u;
    const uint32_t wd = d >> 5, wr = o >> 5;
    const uint32_t l0 = __ballot_sync(kFull, lead_d && wd == 0u), l1 = __ballot_sync(kFull, lead_d && wd == 1u),
                   l2 = __ballot_sync(kFull, lead_d && wd == 2u), r1 = __ballot_sync(kFull, lead_r && wr == 1u),
                   r2 = __ballot_sync(kFull, lead_r && wr == 2u), r3 = __ballot_sync(kFull, lead_r && wr == 3u);
    const uint32_t n0 = __popc(l0), n1 = __popc(l1), n2 = __popc(l2), k1 = __popc(r1), k2 = __popc(r2),
                   k3 = __popc(r3);
    fallback = fallback || n0 > 31u || n1 > 31u || n2 > 31u;  // a run has four bits: k <= 8
    if (!fallback && lead_d && wd < 3u) {
      const uint32_t at = wd == 0u ? __popc(l0 & lt) : wd == 1u ? n0 + __popc(l1 & lt) : n0 + n1 + __popc(l2 & lt);
      st->res_pairs[(size_t)j * kMsb + at] = make_uint2(m, d & 31u);
    }
    if (!fallback && lead_r) {
      const uint32_t c = n0 + n1 + n2;
      const uint32_t at = wr == 1u ? c + __popc(r1 & lt) : wr == 2u ? c + k1 + __popc(r2 & lt)
                                                                  : c + k1 + k2 + __popc(r3 & lt);
      st->res_pairs[(size_t)j * kMsb + at] = make_uint2(ms, 31u - (o & 31u));
    }
    if (lane == 0)
      st->res_cnt[j] = fallback ? 1u << 31 : n0 | n1 << 5 | n2 << 10 | k1 << 15 | k2 << 20 | k3 << 25;
  }
}

// The gather.  A warp takes a unit of kNatGroups consecutive new groups x 64
// consecutive sites, lane = sites t and t + 32: every load and store is a
// coalesced 128-byte row segment, and a group's pair list is the same for
// all lanes (staged in shared memory kNatBatch groups at a time, read as
// broadcasts), so no lane waits for another's longer list.  Units are spread
// over the persistent warps by a grid stride (the batch-wide unit prefix
// gives each population its range).
__device__ __forceinline__ void nat_apply(uint32_t (&out)[2], const uint32_t (&lo)[2], const uint32_t (&hi)[2],
                                          const uint2* pg, int i0, int i1) {
#pragma unroll 1
  for (int i = i0; i < i1; ++i) {
    const uint2 a = pg[i];
    out[0] |= __funnelshift_r(lo[0], hi[0], a.y) & a.x;
    out[1] |= __funnelshift_r(lo[1], hi[1], a.y) & a.x;
  }
}

// broadcast pairs (M, 31 - p): bit p of the window word w, copied to every
// bit of M (the shift left puts bit p on top, the arithmetic shift spreads it)
__device__ __forceinline__ void nat_bcast(uint32_t (&out)[2], const uint32_t (&w)[2], const uint2* pg, int i0,
                                          int i1) {
#pragma unroll 1
  for (int i = i0; i < i1; ++i) {
    const uint2 a = pg[i];
    out[0] |= (uint32_t)((int32_t)(w[0] << a.y) >> 31) & a.x;
    out[1] |= (uint32_t)((int32_t)(w[1] << a.y) >> 31) & a.x;
  }
}

__global__ void __launch_bounds__(kNatThreads, kNatBlocksPerSM) msc_resample_native_kernel(BatchDev* b) {
  __shared__ uint2 s_pairs[kNatThreads / 32][kNatBatch * kMsb];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint2* sp = s_pairs[wid];
  const int total = b->res_prefix[b->npop];
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int u = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; u < total; u += nwarps) {
    int lo = 0, hi = b->npop;  // population of unit u (warp-uniform)
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (b->res_prefix[mid] <= u) lo = mid;
      else hi = mid;
    }
    const PopDev* st = b->pops + lo;
    const int N = st->N, Rn = st->R_cur, rgn = (Rn + kMsb - 1) / kMsb, nstrip = (N + kNatSites - 1) / kNatSites;
    const int loc = u - b->res_prefix[lo], tile = loc / nstrip, strip = loc - tile * nstrip;
    const int j0 = tile * kNatGroups, ng = min(kNatGroups, rgn - j0);
    const int t = strip * kNatSites + lane;
    const bool tv0 = t < N, tv1 = t + 32 < N;
    const uint32_t* old = (const uint32_t*)st->spins[st->parity ^ 1] + t;  // this lane's first site in old group 0
    uint32_t* neu = (uint32_t*)st->spins[st->parity] + t;
    const uint32_t* src = st->src;
    const int gmax = st->rgcap - 1;
    // lane g < ng: count word and window start of group j0 + g
    uint32_t cnt_l = 0u;
    int first_l = 0;
    if (lane < ng) {
      cnt_l = st->res_cnt[j0 + lane];
      first_l = (int)(src[(size_t)(j0 + lane) * kMsb] >> 5);
    }
    if (strip == 0) {  // active flags: lane = bit
      uint8_t* act = st->active[st->parity];
      for (int g = 0; g < ng; ++g) act[(j0 + g) * kMsb + lane] = ((j0 + g) * kMsb + lane) < Rn ? 1 : 0;
    }
#pragma unroll 1
    for (int g0 = 0; g0 < ng; g0 += kNatBatch) {
      const int nbat = min(kNatBatch, ng - g0);
      __syncwarp();  // the previous batch is done with the staged pairs
      {  // pair lists of groups j0+g0 .. (contiguous, kMsb slots each) into shared memory
        const uint4* gp = reinterpret_cast<const uint4*>(st->res_pairs + (size_t)(j0 + g0) * kMsb);
        uint4* s4 = reinterpret_cast<uint4*>(sp);
#pragma unroll
        for (int k = lane; k < kNatBatch * kMsb / 2; k += 32)
          if (k < nbat * kMsb / 2) s4[k] = __ldg(gp + k);
      }
      uint32_t W[kNatBatch][4][2];
#pragma unroll
      for (int g = 0; g < kNatBatch; ++g) {
        const int first = __shfl_sync(kFull, first_l, g0 + g);
        if (g < nbat) {
          // the window's rows (clamped rows are never selected by a mask)
          const bool inside = first >= 1 && first + 2 <= gmax;  // warp-uniform
          const uint32_t* r = old + (size_t)(inside ? first - 1 : 0) * N;
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const uint32_t* rq = inside ? r + (size_t)q * N : old + (size_t)min(max(first - 1 + q, 0), gmax) * N;
            W[g][q][0] = tv0 ? __ldg(rq) : 0u;
            W[g][q][1] = tv1 ? __ldg(rq + 32) : 0u;
          }
        }
      }
      __syncwarp();
#pragma unroll
      for (int g = 0; g < kNatBatch; ++g) {
        if (g >= nbat) break;  // warp-uniform
        const uint32_t cnt = __shfl_sync(kFull, cnt_l, g0 + g);
        const int c1 = cnt & 31u, c2 = c1 + ((cnt >> 5) & 31u), c3 = c2 + ((cnt >> 10) & 31u);
        const int c4 = c3 + ((cnt >> 15) & 31u), c5 = c4 + ((cnt >> 20) & 31u), c6 = c5 + ((cnt >> 25) & 31u);
        const uint2* pg = sp + g * kMsb;
        uint32_t out[2] = {0u, 0u};
        nat_apply(out, W[g][0], W[g][1], pg, 0, c1);
        nat_apply(out, W[g][1], W[g][2], pg, c1, c2);
        nat_apply(out, W[g][2], W[g][3], pg, c2, c3);
        nat_bcast(out, W[g][1], pg, c3, c4);
        nat_bcast(out, W[g][2], pg, c4, c5);
        nat_bcast(out, W[g][3], pg, c5, c6);
        const int j = j0 + g0 + g;
        if (cnt >> 31) {  // sources beyond the window: bit by bit (warp-uniform)
          const int nb = min(kMsb, Rn - j * kMsb);
#pragma unroll 1
          for (int bb = 0; bb < nb; ++bb) {
            const uint32_t lin = src[(size_t)j * kMsb + bb];
            const uint32_t* rl = old + (size_t)(lin >> 5) * N;
            const uint32_t v0 = tv0 ? __ldg(rl) : 0u, v1 = tv1 ? __ldg(rl + 32) : 0u;
            out[0] |= ((v0 >> (lin & 31u)) & 1u) << bb;
            out[1] |= ((v1 >> (lin & 31u)) & 1u) << bb;
          }
        }
        uint32_t* d = neu + (size_t)j * N;
        if (tv0) d[0] = out[0];
        if (tv1) d[32] = out[1];
      }
    }
  }
}

// -------------------------------------------------------------- geometry
// A work unit is a tile of G groups whose lattices are stacked into G*L
// sublattice rows; every pass of a half-sweep updates rpp of those rows with
// Wr threads each.  G is chosen to fill the thread slots of whole kKB-site
// batches: small lattices (L=16: 128 words per half-sweep) would otherwise
// leave most of a 256-thread CTA idle.
static double msc_fill(int L, int G, int* rpp, int* npass) {
  const int Wr = L / 2, VR = G * L;
  int r = kSweepThreads / Wr;
  if (r > VR) r = VR;
  const int np = (VR + r - 1) / r, padded = (np + kKB - 1) / kKB * kKB;
  *rpp = r;
  *npass = np;
  return (double)VR * Wr / ((double)padded * kSweepThreads);
}

bool msc_geom(int L, SweepGeom* g, int tile, long long groups, int slots) {
  if (L < 8 || L % 2 != 0 || L > 128) return false;
  g->L = L;
  g->N = L * L;
  g->half = g->N / 2;
  g->Wr = L / 2;
  // G > 1 moves each sublattice with 16-byte vectors (h % 4 == 0) and keeps
  // the tile small enough for four resident CTAs per SM
  auto allowed = [&](int G) {
    return G == 1 || (G == 2 || G == 4 || G == kMaxTile) && g->half % 4 == 0 && G * g->N * 4 <= kTileSmemMax;
  };
  int best_G = 1, rpp = 0, npass = 0;
  if (tile > 0) {
    if (!allowed(tile)) return false;
    best_G = tile;
  } else if (groups > 0 && slots > 0) {
    // automatic, by a cost model: waves of work units over the resident
    // CTAs times the thread slots one unit occupies per half-sweep (whole
    // kKB-site batches), with the stacking arithmetic of G > 1 counted as
    // 7% more work (the measured gap at equal fill)
    auto cost = [&](int G) {
      int r, np;
      msc_fill(L, G, &r, &np);
      const double waves = std::max(1.0, (double)((groups + G - 1) / G) / slots);
      return waves * ((np + kKB - 1) / kKB * kKB) * (G > 1 ? 1.07 : 1.0);
    };
    double best = cost(1);
    for (int G = 2; G <= kMaxTile; G *= 2) {
      if (!allowed(G)) continue;
      const double c = cost(G);
      if (c < best - 1e-9) {
        best = c;
        best_G = G;
      }
    }
  }
  g->G = best_G;
  msc_fill(L, best_G, &rpp, &npass);
  g->rpp = rpp;
  g->T = g->Wr * rpp;
  g->npass = npass;
  g->kconst = (g->half % kRefThreads == 0) ? g->half / kRefThreads : 0;
  g->smem = best_G == 1 ? (msc_halo_block(L, g->Wr) + (L + 2) * g->Wr) * 4 : best_G * g->N * 4;
  return true;
}

// -------------------------------------------------------------- launchers
int msc_fixed_l(int L, int G) { return G == 1 && L == 96 ? L : 0; }

static const void* msc_sweep_fn(int rng_mode, int fixed_l) {
  if (rng_mode == kRefCoords) return (const void*)msc_sweep_kernel<kRefCoords, 0>;
  return fixed_l == 96         ? (const void*)msc_sweep_kernel<kNative, 96>
         : fixed_l == kWith96 ? (const void*)msc_sweep_kernel<kNative, kWith96>
                              : (const void*)msc_sweep_kernel<kNative, 0>;
}

cudaError_t msc_sweep_setup(int rng_mode, int smem, SweepLaunch* out, int fixed_l) {
  if (rng_mode == kRefCoords || (fixed_l != 96 && fixed_l != kWith96)) fixed_l = 0;
  cudaError_t e = persistent_launch(msc_sweep_fn(rng_mode, fixed_l), kSweepThreads, smem, out);
  out->fixed_l = fixed_l;
  return e;
}

cudaError_t launch_msc_sweep(BatchDev* b, int rng_mode, int energy_only, unsigned long long seed,
                             const SweepLaunch& sl, cudaStream_t s) {
  if (rng_mode == kRefCoords) {
    msc_sweep_kernel<kRefCoords, 0><<<sl.grid, sl.block, sl.smem, s>>>(b, energy_only, seed);
  } else {
    if (sl.fixed_l == 96)
      msc_sweep_kernel<kNative, 96><<<sl.grid, sl.block, sl.smem, s>>>(b, energy_only, seed);
    else if (sl.fixed_l == kWith96)
      msc_sweep_kernel<kNative, kWith96><<<sl.grid, sl.block, sl.smem, s>>>(b, energy_only, seed);
    else
      msc_sweep_kernel<kNative, 0><<<sl.grid, sl.block, sl.smem, s>>>(b, energy_only, seed);
  }
  return cudaGetLastError();
}

cudaError_t launch_msc_init(PopDev* pops, int npop, cudaStream_t s) {
  msc_init_kernel<<<dim3(256, npop), 256, 0, s>>>(pops);
  return cudaGetLastError();
}

cudaError_t launch_msc_resample(BatchDev* b, int rng_mode, cudaStream_t s) {
  int dev, nsm;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  msc_resample_plan_kernel<<<1, 1024, 0, s>>>(b, rng_mode == kNative ? 1 : 0);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if (rng_mode == kRefCoords) {
    msc_resample_kernel<<<nsm * kResampleBlocksPerSM, kResampleThreads, 0, s>>>(b);  // persistent warps
    return cudaGetLastError();
  }
  msc_pairs_kernel<<<nsm * 8, 256, 0, s>>>(b);  // a warp per new group, grid-stride
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  msc_resample_native_kernel<<<nsm * kNatBlocksPerSM, kNatThreads, 0, s>>>(b);
  return cudaGetLastError();
}

}  // namespace pa
