// pa_ssc_bits.cu -- single-spin-coded populations swept on bit planes
// (native stream, L = 64, 128 or 256).
//
// The population stays in the SSC layout in HBM (one int8 +-1 per site,
// sublattice A then B, site (x, y) at idx = y*L/2 + x/2, PAisingSSC.cu:169).
// A CTA loads a tile of G replicas and packs every sublattice row of each
// into L/64 words, bit i = site i of the row (1 == +1): "multi-site coding",
// 32 sites of one replica per word.  In a checkerboard half-sweep the sites of
// one sublattice are independent, so a row word is updated at once: its four
// neighbour words are the other sublattice's rows y-1, y, y+1 and row y
// shifted by one site (towards x-1 or x+1 by row parity, as in
// PAisingSSC.cu:170,182), their anti-parallel counts come from the bitsliced
// adder, and the 32 Metropolis decisions from the digit-serial acceptance of
// the multi-spin-coded sweep (accept_native): each site flips with
// probability exactly min(1, T/2^32), T = ceil(2^32 e^{-beta dE}), the
// thresholds of the int8 sweep.  The energy and magnetisation of each replica
// are population counts of the planes.  The tile is unpacked and written
// back once per temperature.
//
// Work per tile and half-sweep: G * L * L/64 row words = 1024, four per
// thread, decided together (kKB = 4).
#include "pa_kernels.h"
#include "pa_msc_core.cuh"

namespace pa {

using namespace msc;

namespace {

constexpr uint32_t kLsb4 = 0x01010101u;

// bits j of the 4 bytes of w (+1 -> 1, -1 -> 0), j = byte index
__device__ __forceinline__ uint32_t pack4(uint32_t w) {
  const uint32_t plus = ~(w >> 1) & kLsb4;  // +1 = 0x01, -1 = 0xFF
  return (plus * 0x01020408u) >> 24;        // byte j's bit 0 to bit j
}
__device__ __forceinline__ uint32_t pack16(uint4 v) {
  return pack4(v.x) | (pack4(v.y) << 4) | (pack4(v.z) << 8) | (pack4(v.w) << 12);
}
// 4 bits to 4 bytes: bit j set -> +1 (0x01), clear -> -1 (0xFF)
__device__ __forceinline__ uint32_t unpack4(uint32_t n) {
  const uint32_t ones = (n * 0x00204081u) & kLsb4;
  return 0xFFFFFFFFu ^ (ones * 0xFEu);
}
__device__ __forceinline__ uint4 unpack16(uint32_t bits) {
  return make_uint4(unpack4(bits & 0xFu), unpack4((bits >> 4) & 0xFu), unpack4((bits >> 8) & 0xFu),
                    unpack4((bits >> 12) & 0xFu));
}

constexpr int kMaxBitsTile = 16;

}  // namespace

bool ssc_bits_geom(int L, SweepGeom* g) {
  if (L != 64 && L != 128 && L != 256) return false;
  g->L = L;
  g->N = L * L;
  g->half = g->N / 2;
  g->Wr = L / 64;                // words per sublattice row
  const int wpp = L * g->Wr;     // words per sublattice plane
  g->G = 1024 / wpp;             // replicas per tile: 1024 row words per half-sweep
  g->T = kSweepThreads;
  g->rpp = 0;
  g->npass = g->G * wpp / kSweepThreads;  // row words per thread per half-sweep (4)
  g->kconst = 0;
  g->smem = g->G * 2 * wpp * 4;
  return g->G >= 1 && g->G <= kMaxBitsTile;
}

__global__ void __launch_bounds__(kSweepThreads, 4)
    ssc_sweep_bits_kernel(BatchDev* b, int energy_only, unsigned long long stream_seed) {
  extern __shared__ __align__(16) uint32_t pl[];  // [X][g][y][c]: plane X of replica g, row y, word c
  __shared__ int s_unit, s_pop;
  __shared__ uint2 s_dig[kMsb];
  __shared__ int s_anti[kMaxBitsTile], s_plus[kMaxBitsTile];
  __shared__ UnitParams P;
  __shared__ BitStats stats;  // lane g accumulates the replicas in slot g of its tiles

  const int tid = threadIdx.x;
  const int total = b->unit_prefix[b->npop];
  const PhiloxKeys keys(stream_seed);
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
        P.L = st->L; P.N = st->N; P.h = st->N >> 1; P.Wr = st->Wr; P.G = st->gpt;
        P.rg = st->R_cur;  // replicas
        P.step = st->step;
        P.sweeps = energy_only ? 0 : st->sweeps;
        P.tag = kTagSscSweep | (uint32_t)st->pop_id;
        P.T4 = st->thr[(size_t)st->step * kThrPerStep + 10];
        P.T8 = st->thr[(size_t)st->step * kThrPerStep + 11];
        P.words = (uint32_t*)st->spins[st->parity];
        P.E = st->E;
        P.M = st->M;
      }
    }
    if (tid < kMaxBitsTile) { s_anti[tid] = 0; s_plus[tid] = 0; }
    __syncthreads();
    const int p = s_pop, ti = s_unit;
    if (p < 0) break;
    if (p != cur) {  // block-uniform
      if (tid < kMsb && cur >= 0) stats.flush(b->pops + cur, tid);
      cur = p;
      if (tid < kMsb) {
        const uint32_t d4 = 0u - ((P.T4 >> (31 - tid)) & 1u), d8 = 0u - ((P.T8 >> (31 - tid)) & 1u);
        s_dig[tid] = make_uint2(d8, d4 ^ d8);
      }
    }
    const int L = P.L, N = P.N, h = P.h, Wq = P.Wr, G = P.G;
    const int wpp = L * Wq, lwpp = 31 - __clz(wpp), lwq = 31 - __clz(Wq);
    const int r0 = ti * G, gc = min(G, P.rg - r0);
    const uint8_t* spins = (const uint8_t*)P.words;

    // pack: one row word (32 bytes of int8 spins) per item
    for (int it = tid; it < gc * 2 * wpp; it += blockDim.x) {
      const int g = it >> (lwpp + 1), X = (it >> lwpp) & 1, w = it & (wpp - 1);
      const uint4* src = (const uint4*)(spins + (size_t)(r0 + g) * N + (size_t)X * h + (size_t)w * 32);
      pl[(X * G + g) * wpp + w] = pack16(src[0]) | (pack16(src[1]) << 16);
    }
    __syncthreads();

    const int items = gc * wpp;  // row words of one plane present in the tile
    const int sweeps = P.sweeps;
    for (int sw = 0; sw < sweeps; ++sw) {
#pragma unroll 1
      for (int hf = 0; hf < 2; ++hf) {
        uint32_t* self = pl + hf * G * wpp;
        const uint32_t* oth = pl + (1 - hf) * G * wpp;
        const uint32_t c1 = (uint32_t)((sw * 2 + hf) << 4);
#pragma unroll 1
        for (int q0 = 0; q0 * kSweepThreads < G * wpp; q0 += kKB) {
          uint32_t av[kKB], un[kKB], ac[kKB], site[kKB];
          uint32_t vm = 0;
#pragma unroll
          for (int k = 0; k < kKB; ++k) {
            const int it = tid + (q0 + k) * kSweepThreads;
            const bool valid = it < items;
            const int itc = valid ? it : 0;
            const int g = itc >> lwpp, wr = itc & (wpp - 1), y = wr >> lwq, c = wr & (Wq - 1);
            const int base = g * wpp, row = y * Wq;
            const int rowu = (y == 0 ? L - 1 : y - 1) * Wq, rowd = (y + 1 == L ? 0 : y + 1) * Wq;
            const uint32_t s = self[base + wr];
            const uint32_t ctr = oth[base + wr], up = oth[base + rowu + c], dn = oth[base + rowd + c];
            // the other horizontal neighbour: site i-1 or i+1 of the same row
            const bool left = (hf == 0) == ((y & 1) == 0);
            uint32_t side;
            if (left) side = __funnelshift_l(oth[base + row + (c == 0 ? Wq - 1 : c - 1)], ctr, 1);
            else side = __funnelshift_r(ctr, oth[base + row + (c + 1 == Wq ? 0 : c + 1)], 1);
            uint32_t s0, s1, s2;
            adder4(s ^ ctr, s ^ side, s ^ up, s ^ dn, s0, s1, s2);
            av[k] = s0;
            ac[k] = s1 | s2;
            un[k] = valid ? ~(s1 | s2) : 0u;
            vm |= valid ? 1u << k : 0u;
            site[k] = (uint32_t)(r0 + g) * (uint32_t)wpp + (uint32_t)wr;
          }
          const uint32_t chain = ((uint32_t)ti * blockDim.x + (uint32_t)tid) * 8u + (uint32_t)(q0 / kKB);
          accept_native(av, un, ac, site, chain, c1, (uint32_t)P.step, P.tag, keys, s_dig, kKB);
#pragma unroll
          for (int k = 0; k < kKB; ++k)
            if (vm >> k & 1u) {
              const int it = tid + (q0 + k) * kSweepThreads;
              self[(it >> lwpp) * wpp + (it & (wpp - 1))] ^= ac[k];
            }
        }
        __syncthreads();
      }
    }

    // energy (every bond seen once from its A end: E = -2N + 2 #anti-parallel)
    // and magnetisation (M = 2 #plus - N) of each replica of the tile
    for (int it = tid; it < items; it += blockDim.x) {
      const int g = it >> lwpp, wr = it & (wpp - 1), y = wr >> lwq, c = wr & (Wq - 1);
      const int base = g * wpp, row = y * Wq;
      const uint32_t* A = pl;
      const uint32_t* B = pl + G * wpp;
      const uint32_t a = A[base + wr], ctr = B[base + wr];
      const uint32_t up = B[base + (y == 0 ? L - 1 : y - 1) * Wq + c], dn = B[base + (y + 1 == L ? 0 : y + 1) * Wq + c];
      const uint32_t side = (y & 1) == 0 ? __funnelshift_l(B[base + row + (c == 0 ? Wq - 1 : c - 1)], ctr, 1)
                                         : __funnelshift_r(ctr, B[base + row + (c + 1 == Wq ? 0 : c + 1)], 1);
      atomicAdd(&s_anti[g], __popc(a ^ ctr) + __popc(a ^ side) + __popc(a ^ up) + __popc(a ^ dn));
      atomicAdd(&s_plus[g], __popc(a) + __popc(ctr));
    }
    // unpack and write the tile back
    uint8_t* dst = (uint8_t*)P.words;
    for (int it = tid; it < gc * 2 * wpp; it += blockDim.x) {
      const int g = it >> (lwpp + 1), X = (it >> lwpp) & 1, w = it & (wpp - 1);
      const uint32_t bits = pl[(X * G + g) * wpp + w];
      uint4* o = (uint4*)(dst + (size_t)(r0 + g) * N + (size_t)X * h + (size_t)w * 32);
      o[0] = unpack16(bits & 0xFFFFu);
      o[1] = unpack16(bits >> 16);
    }
    __syncthreads();
    if (tid < gc) {
      const int E = -2 * N + 2 * s_anti[tid], Mg = 2 * s_plus[tid] - N;
      P.E[r0 + tid] = E;
      P.M[r0 + tid] = Mg;
      stats.add(tid, E, Mg);
    }
  }
  if (tid < kMsb && cur >= 0) stats.flush(b->pops + cur, tid);
}

cudaError_t ssc_bits_setup(int smem, SweepLaunch* out) {
  return persistent_launch((const void*)ssc_sweep_bits_kernel, kSweepThreads, smem, out);
}

cudaError_t launch_ssc_bits_sweep(BatchDev* b, int energy_only, unsigned long long seed, const SweepLaunch& sl,
                                  cudaStream_t s) {
  ssc_sweep_bits_kernel<<<sl.grid, sl.block, sl.smem, s>>>(b, energy_only, seed);
  return cudaGetLastError();
}

}  // namespace pa
