// pa_ssc.cu -- single-spin coding (one int8 +-1 per site).
//
// Replaces, from the reference PAisingSSC.cu:
//   ReplicaInit   (PAisingSSC.cu:150-157)  -> ssc_init_kernel
//   checkKerALL   (PAisingSSC.cu:159-193)  -> ssc_sweep_kernel (all sweeps of a
//   energyKer     (PAisingSSC.cu:195-215)     replica in shared memory, energy
//                                             and magnetisation fused at the end)
//   resampleKer   (PAisingSSC.cu:272-280)  -> ssc_resample_kernel (gather into
//                                             the other half of a double buffer)
//
// Layout in HBM: replica r occupies N bytes at spins + r*N, sublattice A
// (sites with x+y even) first, then B; inside a sublattice, site (x, y) is at
// idx = y*L/2 + x/2, the reference's checkerboard index (PAisingSSC.cu:169).
#include <climits>

#include "pa_device.cuh"
#include "pa_kernels.h"

namespace pa {

namespace {

constexpr uint32_t kLsb = 0x01010101u;

__device__ __forceinline__ uint32_t minus_bits(uint32_t w) { return (w >> 1) & kLsb; }  // 1 per byte == -1

// per-replica statistics kept by thread 0 of a sweep CTA until the CTA moves
// to another population or finishes
struct StatAcc {
  long long sE, sE2, sM, sM2;
  U128 m4;
  int emin;
  __device__ void reset() {
    sE = sE2 = sM = sM2 = 0;
    m4 = U128{0, 0};
    emin = INT_MAX;
  }
  __device__ void add(int e, int m) {
    const long long am = m < 0 ? -(long long)m : (long long)m;
    sE += e;
    sE2 += (long long)e * e;
    sM += am;
    sM2 += am * am;
    unsigned long long lo, hi;
    m4_of(m, lo, hi);
    u128_add(m4, lo, hi);
    emin = e < emin ? e : emin;
  }
  __device__ void flush(PopDev* st) const {
    if (emin == INT_MAX) return;
    atomicAdd((unsigned long long*)&st->sE, (unsigned long long)sE);
    atomicAdd((unsigned long long*)&st->sE2, (unsigned long long)sE2);
    atomicAdd((unsigned long long*)&st->sM, (unsigned long long)sM);
    atomicAdd((unsigned long long*)&st->sM2, (unsigned long long)sM2);
    u128_atomic_add(&st->sM4lo, &st->sM4hi, m4.lo, m4.hi);
    atomicMin(&st->Emin_acc, emin);
  }
};

}  // namespace

// ------------------------------------------------------------------ init
// ReplicaInit (PAisingSSC.cu:150-157): reference thread t of block B draws,
// for its k-th site idx = t + 128k, uniform number 2k for gA[idx] and 2k+1
// for gB[idx] from subsequence iseq + t + 128 B; spin = +1 iff U >= 0.5.
__global__ void ssc_init_kernel(PopDev* pops) {
  PopDev* st = pops + blockIdx.y;
  const int N = st->N, h = N >> 1, R = st->R_cur;
  const unsigned long long seed = st->seed, iseq = st->iseq;
  int8_t* sp = (int8_t*)st->spins[st->parity];
  if (st->init_src) {  // caller-supplied population: copy, 16 bytes per thread
    const uint4* src = (const uint4*)st->init_src;
    uint4* dst = (uint4*)sp;
    const long long nv = (long long)R * N / 16;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nv; v += (long long)gridDim.x * blockDim.x)
      dst[v] = src[v];
    return;
  }
  const long long total = (long long)R * h;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(e / h), idx = (int)(e - (long long)r * h);
    const int t = idx & (kRefThreads - 1), k = idx >> 7;
    const unsigned long long sub = iseq + (unsigned long long)t + (unsigned long long)kRefThreads * r;
    sp[(size_t)r * N + idx] = ref_uniform(ref_word(seed, sub, 2ull * k)) >= 0.5 ? 1 : -1;
    sp[(size_t)r * N + h + idx] = ref_uniform(ref_word(seed, sub, 2ull * k + 1)) >= 0.5 ? 1 : -1;
  }
}

// ----------------------------------------------------------------- sweep
// Persistent: every CTA takes replicas of any population from the batch's
// work queue and anneals one replica at a time, the whole lattice resident in
// shared memory as 32-bit words of 4 int8 spins.  Thread (rsub, cw) owns word
// column cw of sublattice rows rsub, rsub+rpp, ...
//
// MODE kRefCoords reproduces checkKerALL's decisions exactly: site idx of
// replica r, sweep sw, half-sweep hf uses draw
//     ctr = sw*2K + hf*K + k   of subsequence  iseq + t + 128 r,
// t = idx mod 128, k = idx div 128, K = draws per reference thread per half
// sweep, and flips iff (H+1)/2^32 < boltz[idxT0 + 2 idxT1], evaluated as the
// integer test H < thr10[...] with thr10 = ceil(2^32 p) - 1 (exact).
// MODE kNative flips iff dE <= 0 or U < T = ceil(2^32 exp(-beta dE)) for a
// uniform 32-bit U, decided one byte at a time: U's top byte b against T's
// top byte t settles the test unless b == t (probability 1/256), and only
// then are U's low 24 bits drawn and compared with T's.  One Philox4x32-10
// block serves two words (8 sites): words x, y give the top bytes, z, w the
// low bits of up to two undecided sites; more than two take another block.
// Each site's acceptance probability is exactly T / 2^32.
template <int MODE>
__global__ void __launch_bounds__(kSweepThreads, 4)
    ssc_sweep_kernel(BatchDev* b, int energy_only, unsigned long long stream_seed) {
  extern __shared__ __align__(16) uint32_t lat[];  // N/4 words: A then B
  __shared__ uint32_t s_thr[16];
  __shared__ int s_unit, s_pop;
  __shared__ int s_red[2][33];

  const int tid = threadIdx.x;
  const int total = b->unit_prefix[b->npop];
  int cur = -1;
  PopDev* st = nullptr;
  int L = 0, N = 0, h = 0, Wr = 1, hw = 0, rpp = 1, kconst = 0, step = 0, sweeps = 0;
  uint32_t nstep = 0;  // counter word 2 of the native stream
  unsigned long long seed = 0, iseq = 0;
  // native stream key: one seed for the whole batch; populations differ in counter word 3
  const uint32_t k0 = (uint32_t)stream_seed, k1 = (uint32_t)(stream_seed >> 32);
  uint32_t tag = 0;
  int8_t* spins = nullptr;
  bool worker = false;
  int cw = 0, rsub = 0, cwl = 0, cwr = 0;
  StatAcc acc;
  acc.reset();

  for (;;) {
    __syncthreads();
    if (tid == 0) {
      const int u = (int)atomicAdd(&b->work_next, 1u);
      int loc = 0;
      s_pop = u < total ? queue_pop(b, u, &loc) : -1;
      s_unit = loc;
    }
    __syncthreads();
    const int p = s_pop, r = s_unit;
    if (p < 0) break;
    if (p != cur) {  // block-uniform: load the population's parameters
      if (tid == 0 && st) {
        acc.flush(st);
        acc.reset();
      }
      cur = p;
      st = b->pops + p;
      L = st->L; N = st->N; h = N >> 1; hw = h >> 2; Wr = st->Wr; rpp = st->rpp; kconst = st->kconst;
      step = st->step;
      nstep = native_step_word(st);
      sweeps = energy_only ? 0 : st->sweeps;
      seed = st->seed;
      tag = kTagSscSweep | (uint32_t)st->pop_id;
      // draws consumed by the resampling of this step come before the sweep's
      iseq = st->iseq + (step > 0 ? (unsigned long long)st->R_prev : 0ull);
      spins = (int8_t*)st->spins[st->parity];
      worker = tid < st->T;
      cw = worker ? tid % Wr : 0;
      rsub = worker ? tid / Wr : 0;
      cwl = (cw == 0 ? Wr - 1 : cw - 1);
      cwr = (cw + 1 == Wr ? 0 : cw + 1);
      if (tid < kThrPerStep) s_thr[tid] = st->thr[(size_t)step * kThrPerStep + tid];
    }
    const uint4* gsrc = (const uint4*)(spins + (size_t)r * N);
    uint4* lat4 = (uint4*)lat;
    for (int v = tid; v < (N >> 4); v += blockDim.x) lat4[v] = gsrc[v];
    __syncthreads();

    for (int sw = 0; sw < sweeps; ++sw) {
#pragma unroll 1
      for (int hf = 0; hf < 2; ++hf) {
        uint32_t* self = lat + (hf ? hw : 0);
        const uint32_t* oth = lat + (hf ? 0 : hw);
        // anti-parallel neighbour count (0..4) of each of the 4 sites of word
        // (ty, cw); the horizontal neighbour that is not at the same idx is x-1
        // for A on even rows and B on odd rows, x+1 otherwise (PAisingSSC.cu:170,182)
        auto anti = [&](int ty, const uint32_t* oth, uint32_t s, int hf_) {
          const int row = ty * Wr, rowu = (ty == 0 ? L - 1 : ty - 1) * Wr, rowd = (ty + 1 == L ? 0 : ty + 1) * Wr;
          const uint32_t o = oth[row + cw];
          const bool left = (hf_ == 0) == ((ty & 1) == 0);
          const uint32_t oside = left ? __byte_perm(oth[row + cwl], o, 0x6543) : __byte_perm(o, oth[row + cwr], 0x4321);
          const uint32_t ou = oth[rowu + cw], od = oth[rowd + cw];
          return ((s ^ o) >> 1 & kLsb) + ((s ^ oside) >> 1 & kLsb) + ((s ^ ou) >> 1 & kLsb) + ((s ^ od) >> 1 & kLsb);
        };
        if (worker && MODE == kNative) {
          const uint32_t T4 = s_thr[10], T8 = s_thr[11];
          const uint32_t t4b = (T4 >> 24) * kLsb, t8b = (T8 >> 24) * kLsb;
          const uint32_t c1 = (uint32_t)(sw * 2 + hf) * 2u;
          for (int ty0 = rsub; ty0 < L; ty0 += 2 * rpp) {
            const int ty1 = ty0 + rpp;
            const bool two = ty1 < L;
            const int w0 = ty0 * Wr + cw, w1 = two ? ty1 * Wr + cw : w0;
            uint32_t s[2], na[2], flip[2], strag[2];
            s[0] = self[w0];
            s[1] = self[w1];
            na[0] = anti(ty0, oth, s[0], hf);
            na[1] = two ? anti(ty1, oth, s[1], hf) : 0x02020202u;  // no decision needed
            const U4 rn = philox10((uint32_t)(r * hw + w0), c1, nstep, tag, k0, k1);
            const uint32_t top[2] = {rn.x, rn.y};
#pragma unroll
            for (int q = 0; q < 2; ++q) {
              const uint32_t one = __vcmpeq4(na[q], kLsb), need = __vcmpleu4(na[q], kLsb);
              const uint32_t tb = (t4b & one) | (t8b & ~one);  // T's top byte per site
              flip[q] = (~need | (need & __vcmpltu4(top[q], tb))) & 0xFEFEFEFEu;
              strag[q] = need & __vcmpeq4(top[q], tb);  // top bytes equal: undecided
            }
            if (strag[0] | strag[1]) {  // probability ~ 2/256 per site needing a decision
              // undecided sites as bits q*4 + j; their low 24 bits come from
              // rn.z, rn.w, then from further blocks, four words each
              uint32_t pend = (((strag[0] & kLsb) * 0x01020408u) >> 24) | ((((strag[1] & kLsb) * 0x01020408u) >> 24) << 4);
              uint32_t a0 = rn.z, a1 = rn.w, a2 = 0u, a3 = 0u, fl = 0u;
              int used = 0;
#pragma unroll 1
              while (pend) {
                const int bit = __ffs(pend) - 1;
                pend &= pend - 1;
                if (used == 2 || used == 6) {
                  const U4 x = philox10((uint32_t)(r * hw + w0), c1 + 1u, nstep,
                                        tag | ((uint32_t)(used >> 2) << 12), k0, k1);
                  a0 = x.x; a1 = x.y; a2 = x.z; a3 = x.w;
                }
                const int slot = used < 2 ? used : (used - 2) & 3;
                const uint32_t u = slot == 0 ? a0 : slot == 1 ? a1 : slot == 2 ? a2 : a3;
                ++used;
                const uint32_t nq = bit < 4 ? na[0] : na[1];
                const uint32_t T = ((nq >> (8 * (bit & 3))) & 0xFFu) == 1u ? T4 : T8;
                if ((u & 0xFFFFFFu) < (T & 0xFFFFFFu)) fl |= 1u << bit;
              }
#pragma unroll
              for (int j = 0; j < 4; ++j) {
                flip[0] |= ((fl >> j) & 1u) ? 0xFEu << (8 * j) : 0u;
                flip[1] |= ((fl >> (4 + j)) & 1u) ? 0xFEu << (8 * j) : 0u;
              }
            }
            self[w0] = s[0] ^ flip[0];
            if (two) self[w1] = s[1] ^ flip[1];
          }
        }
        if (worker && MODE == kRefCoords) {
          for (int ty = rsub; ty < L; ty += rpp) {
            const int row = ty * Wr, rowu = (ty == 0 ? L - 1 : ty - 1) * Wr, rowd = (ty + 1 == L ? 0 : ty + 1) * Wr;
            const int w = row + cw;
            const uint32_t s = self[w];
            const uint32_t o = oth[w];
            const bool left = (hf == 0) == ((ty & 1) == 0);
            const uint32_t oside = left ? __byte_perm(oth[row + cwl], o, 0x6543) : __byte_perm(o, oth[row + cwr], 0x4321);
            const uint32_t ou = oth[rowu + cw], od = oth[rowd + cw];
            uint32_t flip = 0;
            {
              const uint32_t nminus = minus_bits(o) + minus_bits(oside) + minus_bits(ou) + minus_bits(od);
              // idxT0 + 2 idxT1 = (1 - s_minus) + 2 (4 - n_minus) per byte
              const uint32_t tix = 0x09090909u - minus_bits(s) - (nminus << 1);
              const int idx0 = ty * (h / L) + cw * 4;
#pragma unroll
              for (int j = 0; j < 4; ++j) {
                const int idx = idx0 + j, t = idx & (kRefThreads - 1), k = idx >> 7;
                const int K = kconst ? kconst : (t < h ? (h - t + kRefThreads - 1) / kRefThreads : 0);
                const unsigned long long sub = iseq + (unsigned long long)t + (unsigned long long)kRefThreads * r;
                const unsigned long long ctr = (unsigned long long)sw * 2 * K + (unsigned long long)hf * K + k;
                const uint32_t u = ref_word(seed, sub, ctr);
                if (u < s_thr[(tix >> (8 * j)) & 0xFFu]) flip |= 0xFEu << (8 * j);
              }
            }
            self[w] = s ^ flip;
          }
        }
        __syncthreads();
      }
    }

    // energy: every bond joins one A and one B site, so E = -sum_A s_A sum_nn s_B
    // = -2N + 2 * (number of anti-parallel bonds seen from A); M = N - 2 #minus.
    int anti = 0, nminus = 0;
    if (worker) {
      for (int ty = rsub; ty < L; ty += rpp) {
        const int row = ty * Wr, rowu = (ty == 0 ? L - 1 : ty - 1) * Wr, rowd = (ty + 1 == L ? 0 : ty + 1) * Wr;
        const int w = row + cw;
        const uint32_t s = lat[w], o = lat[hw + w];
        const bool left = (ty & 1) == 0;
        const uint32_t oside = left ? __byte_perm(lat[hw + row + cwl], o, 0x6543) : __byte_perm(o, lat[hw + row + cwr], 0x4321);
        const uint32_t na = ((s ^ o) >> 1 & kLsb) + ((s ^ oside) >> 1 & kLsb) + ((s ^ lat[hw + rowu + cw]) >> 1 & kLsb) +
                            ((s ^ lat[hw + rowd + cw]) >> 1 & kLsb);
        anti += (int)((na * kLsb) >> 24);
        nminus += __popc(minus_bits(s)) + __popc(minus_bits(o));
      }
    }
    anti = warp_sum(anti);
    nminus = warp_sum(nminus);
    if ((tid & 31) == 0) { s_red[0][tid >> 5] = anti; s_red[1][tid >> 5] = nminus; }
    // write the lattice back while the reduction completes
    uint4* gdst = (uint4*)(spins + (size_t)r * N);
    __syncthreads();
    for (int v = tid; v < (N >> 4); v += blockDim.x) gdst[v] = lat4[v];
    if (tid == 0) {
      int a = 0, m = 0;
      for (int i = 0; i < (int)(blockDim.x >> 5); ++i) { a += s_red[0][i]; m += s_red[1][i]; }
      const int E = -2 * N + 2 * a, Mg = N - 2 * m;
      st->E[r] = E;
      st->M[r] = Mg;
      acc.add(E, Mg);
    }
  }
  if (tid == 0 && st) acc.flush(st);
}

// -------------------------------------------------------------- resample
// Gather form of resampleKer: new replica s copies old replica src[s].
//
// Work unit: up to kSscUnitVecs 16-byte vectors of one population's new
// buffer -- whole replicas (floor(kSscUnitVecs / nv) of them) when a replica
// has at most kSscUnitVecs vectors, else one kSscUnitVecs part of a replica.
// Units of all populations of the batch come from one queue
// (ssc_resample_plan_kernel) and are taken by persistent CTAs, so a batch of
// uneven populations keeps every SM copying until the last unit; each thread
// issues all its loads of a unit before its stores.
constexpr int kSscResThreads = 256;
constexpr int kSscVecsPerThread = 8;
constexpr int kSscUnitVecs = kSscResThreads * kSscVecsPerThread;  // 32 KB
constexpr int kSscResBlocksPerSM = 4;  // 64 registers

__host__ __device__ __forceinline__ long long ssc_units(int nv, int Rn) {
  if (nv > kSscUnitVecs) return (long long)Rn * ((nv + kSscUnitVecs - 1) / kSscUnitVecs);
  const int rpu = kSscUnitVecs / nv;
  return (Rn + rpu - 1) / rpu;
}

__global__ void __launch_bounds__(1024) ssc_resample_plan_kernel(BatchDev* b) {
  __shared__ uint32_t s_u[33];
  const int p = threadIdx.x, np = b->npop;
  uint32_t units = 0;
  if (p < np) {
    const PopDev* st = b->pops + p;
    if (st->coding == kSSC && pop_stepping(st)) units = (uint32_t)ssc_units(st->N >> 4, st->R_cur);
  }
  uint32_t total;
  const uint32_t ex = block_exscan(units, s_u, &total);
  if (p < np) b->res_prefix[p] = (int)ex;
  if (p == 0) {
    b->res_prefix[np] = (int)total;
    b->res_next = 0;
  }
}

__global__ void __launch_bounds__(kSscResThreads, kSscResBlocksPerSM) ssc_resample_kernel(BatchDev* b) {
  __shared__ int s_u[2];  // this unit and the next one (taken ahead by thread 0)
  const int tid = threadIdx.x, total = b->res_prefix[b->npop];
  if (tid == 0) s_u[0] = (int)atomicAdd(&b->res_next, 1u);
  __syncthreads();
  for (int it = 0;; ++it) {
    const int u = s_u[it & 1];
    if (u >= total) break;  // block-uniform
    if (tid == 0) s_u[(it + 1) & 1] = (int)atomicAdd(&b->res_next, 1u);
    int lo = 0, hi = b->npop;  // population of unit u
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (b->res_prefix[mid] <= u) lo = mid;
      else hi = mid;
    }
    const PopDev* st = b->pops + lo;
    const int nv = st->N >> 4, Rn = st->R_cur, loc = u - b->res_prefix[lo];
    const uint4* old = (const uint4*)st->spins[st->parity ^ 1];
    uint4* neu = (uint4*)st->spins[st->parity];
    const uint32_t* src = st->src;
    // the unit as replicas [s0, s0 + ns) x vectors [j0, j0 + nj) of each
    int s0, ns, j0, nj;
    if (nv > kSscUnitVecs) {
      const int upr = (nv + kSscUnitVecs - 1) / kSscUnitVecs, part = loc % upr;
      s0 = loc / upr;
      ns = 1;
      j0 = part * kSscUnitVecs;
      nj = min(kSscUnitVecs, nv - j0);
    } else {
      const int rpu = kSscUnitVecs / nv;
      s0 = loc * rpu;
      ns = min(rpu, Rn - s0);
      j0 = 0;
      nj = nv;
    }
    const int n = ns * nj;                     // vectors in the unit (<= kSscUnitVecs)
    const uint32_t inv = 0xffffffffu / (uint32_t)nj + 1u;  // n / nj by __umulhi: n * nj < 2^32
    // vector i of the unit is vector j0 + i % nj of new replica s0 + i / nj
    auto at = [&](int i, int& s) {
      const int q = ns == 1 ? 0 : (int)__umulhi((uint32_t)i, inv);
      s = s0 + q;
      return j0 + i - q * nj;
    };
    uint4 r[kSscVecsPerThread];
#pragma unroll
    for (int k = 0; k < kSscVecsPerThread; ++k) {
      const int i = tid + k * kSscResThreads;
      if (i < n) {
        int s;
        const int j = at(i, s);
        r[k] = __ldg(old + (size_t)src[s] * nv + j);
      }
    }
#pragma unroll
    for (int k = 0; k < kSscVecsPerThread; ++k) {
      const int i = tid + k * kSscResThreads;
      if (i < n) {
        int s;
        const int j = at(i, s);
        neu[(size_t)s * nv + j] = r[k];
      }
    }
    __syncthreads();  // s_u[(it + 1) & 1] is visible; s_u[it & 1] may be overwritten
  }
}

// -------------------------------------------------------------- geometry
static int pick_rpp(int L, int Wr) {
  int best = 1;
  for (int r = 1; r <= L; ++r)
    if (L % r == 0 && Wr * r <= kSweepThreads) best = r;
  return best;
}

bool ssc_geom(int L, SweepGeom* g) {
  if (L < 8 || L % 8 != 0 || L > 256) return false;
  g->L = L;
  g->N = L * L;
  g->half = g->N / 2;
  g->Wr = L / 8;
  g->rpp = pick_rpp(L, g->Wr);
  g->T = g->Wr * g->rpp;
  g->npass = (L + g->rpp - 1) / g->rpp;
  g->kconst = (g->half % kRefThreads == 0) ? g->half / kRefThreads : 0;
  g->smem = g->N;
  return true;
}

// -------------------------------------------------------------- launchers
static const void* ssc_sweep_fn(int rng_mode) {
  return rng_mode == kRefCoords ? (const void*)ssc_sweep_kernel<kRefCoords> : (const void*)ssc_sweep_kernel<kNative>;
}

cudaError_t ssc_sweep_setup(int rng_mode, int smem, SweepLaunch* out) {
  return persistent_launch(ssc_sweep_fn(rng_mode), kSweepThreads, smem, out);
}

cudaError_t launch_ssc_sweep(BatchDev* b, int rng_mode, int energy_only, unsigned long long seed,
                             const SweepLaunch& sl, cudaStream_t s) {
  if (rng_mode == kRefCoords)
    ssc_sweep_kernel<kRefCoords><<<sl.grid, sl.block, sl.smem, s>>>(b, energy_only, seed);
  else
    ssc_sweep_kernel<kNative><<<sl.grid, sl.block, sl.smem, s>>>(b, energy_only, seed);
  return cudaGetLastError();
}

cudaError_t launch_ssc_init(PopDev* pops, int npop, cudaStream_t s) {
  ssc_init_kernel<<<dim3(512, npop), 256, 0, s>>>(pops);
  return cudaGetLastError();
}

cudaError_t launch_ssc_resample(BatchDev* b, cudaStream_t s) {
  int dev, nsm;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  ssc_resample_plan_kernel<<<1, 1024, 0, s>>>(b);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  ssc_resample_kernel<<<nsm * kSscResBlocksPerSM, kSscResThreads, 0, s>>>(b);  // persistent CTAs
  return cudaGetLastError();
}

}  // namespace pa
